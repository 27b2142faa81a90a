// bulk_functor.h -- per-voxel bulk source/sink rates of the host mirror
// (reactions-diffusion/biofvm/include/biofvm/bulk_functor.h:8-14).
#pragma once

#include "types.h"

namespace physicore::biofvm {

struct bulk_functor
{
	virtual real_t supply_rates(index_t s, index_t x, index_t y, index_t z) = 0;
	virtual real_t uptake_rates(index_t s, index_t x, index_t y, index_t z) = 0;
	virtual real_t supply_target_densities(index_t s, index_t x, index_t y, index_t z) = 0;
	virtual ~bulk_functor() = default;
};

} // namespace physicore::biofvm
