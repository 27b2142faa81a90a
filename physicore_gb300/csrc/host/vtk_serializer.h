// vtk_serializer.h -- the microenvironment's densities as VTK XML image files, one
// per call, plus a ParaView collection, written without the VTK library.
//
// Output as in the reference (reactions-diffusion/biofvm/src/vtk_serializer.cpp:
// 14-79, vtk_serializer_base.cpp:10-35): <output_dir>/vtk_microenvironment/
// microenvironment_NNNNNN.vti (six-digit call counter), and
// <output_dir>/microenvironment.pvd listing every file written with its time.
// The image's extent starts at bounding_box_min / voxel per axis (integer
// division) and spans the grid; spacing is the voxel shape (z extent 0..0 and
// spacing 0 for a 2-D mesh); one Float64 cell array per density, named after it.
// Arrays are raw appended binary (little-endian, UInt64 size headers).
//
// The densities come from one bulk device-to-host copy in planar order when the
// solver is a gb300_solver (the reference reads every value through a virtual
// get_substrate_density call); other solvers are read value by value.
#pragma once

#include <string>
#include <string_view>
#include <vector>

#include "serializer.h"
#include "types.h"

namespace physicore::biofvm {

struct microenvironment;

class vtk_serializer : public serializer
{
public:
	vtk_serializer(std::string_view output_dir, const microenvironment& m);

	void serialize(const microenvironment& m, real_t current_time) override;

	// Path of the last file written (empty before the first call).
	const std::string& last_file() const { return last_file_; }

private:
	void append_to_pvd(const std::string& file_name, real_t current_time);

	std::size_t iteration_ = 0;
	std::string output_dir_, vtks_dir_, pvd_contents_, last_file_;
	std::string header_; // the file up to the first array's data
	long long extent_[6];
	double spacing_[3];
	std::vector<real_t> planar_; // staging: [s][z][y][x]
};

} // namespace physicore::biofvm
