// agent_data.h -- agent structure-of-arrays of the host mirror, the fields the
// reaction-diffusion step reads (common/include/common/base_agent_data.h positions,
// reactions-diffusion/biofvm/include/biofvm/agent_data_generic_storage.h:16-31).
#pragma once

#include <cstdint>
#include <vector>

#include "types.h"

namespace physicore::biofvm {

struct agent_data
{
	index_t dims = 3;
	index_t substrate_count = 1;
	index_t agents_count = 0;

	std::vector<real_t> positions; // n * dims

	// n * substrate_count
	std::vector<real_t> secretion_rates;
	std::vector<real_t> saturation_densities;
	std::vector<real_t> uptake_rates;
	std::vector<real_t> net_export_rates;
	std::vector<real_t> internalized_substrates;
	std::vector<real_t> fraction_released_at_death;

	std::vector<real_t> volumes;    // n
	std::vector<std::uint8_t> is_active; // n, 1 = active

	agent_data(index_t dims, index_t substrate_count) : dims(dims), substrate_count(substrate_count) {}

	// Appends an agent with zero rates, as agent_data_generic_storage::add does.
	index_t add()
	{
		++agents_count;
		positions.resize(agents_count * dims);
		for (auto* v : { &secretion_rates, &saturation_densities, &uptake_rates, &net_export_rates,
						 &internalized_substrates, &fraction_released_at_death })
			v->resize(agents_count * substrate_count);
		volumes.resize(agents_count);
		is_active.resize(agents_count, 1);
		return agents_count - 1;
	}
};

} // namespace physicore::biofvm
