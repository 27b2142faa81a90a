// mesh.h -- cartesian mesh of the host mirror (reactions-diffusion/biofvm/include/
// biofvm/mesh.h:11-32, src/mesh.cpp:8-77): grid sides are ceil(extent / voxel) on
// the first `dims` axes and 1 on the others; a position maps to its voxel by
// truncating (p - min) / voxel per axis.
#pragma once

#include <array>
#include <cmath>
#include <cstddef>
#include <span>
#include <stdexcept>

#include "types.h"

namespace physicore::biofvm {

struct cartesian_mesh
{
	index_t dims; // 1, 2 or 3

	std::array<sindex_t, 3> bounding_box_mins;
	std::array<sindex_t, 3> bounding_box_maxs;

	std::array<index_t, 3> voxel_shape;
	std::array<index_t, 3> grid_shape;

	cartesian_mesh(index_t dims, std::array<sindex_t, 3> mins, std::array<sindex_t, 3> maxs,
				   std::array<index_t, 3> voxel)
		: dims(dims), bounding_box_mins(mins), bounding_box_maxs(maxs), voxel_shape(voxel), grid_shape { 1, 1, 1 }
	{
		if (dims < 1 || dims > 3)
			throw std::invalid_argument("mesh dims must be 1, 2 or 3");
		for (index_t a = 0; a < dims; a++)
		{
			if (maxs[a] <= mins[a] || voxel[a] == 0)
				throw std::invalid_argument("mesh extent and voxel shape must be positive");
			const index_t extent = (index_t)(maxs[a] - mins[a]);
			grid_shape[a] = (extent + voxel[a] - 1) / voxel[a];
		}
	}

	std::size_t voxel_count() const { return grid_shape[0] * grid_shape[1] * grid_shape[2]; }

	index_t voxel_volume() const { return voxel_shape[0] * voxel_shape[1] * voxel_shape[2]; }

	std::size_t linearize(index_t x, index_t y, index_t z) const
	{
		return x + grid_shape[0] * (y + grid_shape[1] * z);
	}

	std::array<index_t, 3> voxel_position(std::span<const real_t> position) const
	{
		std::array<index_t, 3> v { 0, 0, 0 };
		for (index_t a = 0; a < dims; a++)
			v[a] = (index_t)((position[a] - (real_t)bounding_box_mins[a]) / (real_t)voxel_shape[a]);
		return v;
	}
};

} // namespace physicore::biofvm
