// gb300_solver.cpp -- see gb300_solver.h.
#include "gb300_solver.h"

#include <stdexcept>
#include <string>

#include "solver_registry.h"

namespace physicore::biofvm::kernels::gb300_solver {

namespace {
void check(int rc)
{
	if (rc != PCG_OK)
		throw std::runtime_error(std::string("gb300_solver: ") + pcg_last_error());
}
} // namespace

gb300_solver::~gb300_solver() { pcg_destroy(ctx_); }

std::size_t gb300_solver::index(index_t s, index_t x, index_t y, index_t z) const
{
	return s + S_ * (x + n_[0] * (y + n_[1] * z));
}

void gb300_solver::upload_dirichlet(microenvironment& m)
{
	const index_t S = m.substrates_count;
	std::vector<std::uint8_t> conds(m.dirichlet_interior_voxels_count * S);
	for (std::size_t i = 0; i < conds.size(); i++)
		conds[i] = m.dirichlet_interior_conditions[i] ? 1 : 0;
	check(pcg_set_dirichlet_interior(ctx_, m.dirichlet_interior_voxels_count, m.dirichlet_interior_voxels.get(),
									 m.dirichlet_interior_values.get(), conds.data()));
	std::vector<std::uint8_t> fc(S);
	for (int a = 0; a < 3; a++)
		for (int side = 0; side < 2; side++)
		{
			const real_t* v = (side ? m.dirichlet_max_boundary_values : m.dirichlet_min_boundary_values)[a].get();
			const bool* c = (side ? m.dirichlet_max_boundary_conditions : m.dirichlet_min_boundary_conditions)[a].get();
			if (v && c)
				for (index_t s = 0; s < S; s++)
					fc[s] = c[s] ? 1 : 0;
			check(pcg_set_dirichlet_boundary(ctx_, a, side, v && c ? v : nullptr, v && c ? fc.data() : nullptr));
		}
}

void gb300_solver::upload_agents(microenvironment& m)
{
	if (!m.agents || m.agents->agents_count == 0)
		return;
	agent_data& d = *m.agents;
	check(pcg_set_agents(ctx_, d.agents_count, d.positions.data(), d.secretion_rates.data(),
						 d.saturation_densities.data(), d.uptake_rates.data(), d.net_export_rates.data(),
						 d.volumes.data(), d.is_active.data(), d.internalized_substrates.data(),
						 d.fraction_released_at_death.data(), m.compute_internalized_substrates ? 1 : 0));
	agents_uploaded_ = d.agents_count;
}

void gb300_solver::refresh_agents(microenvironment& m)
{
	const index_t A = m.agents ? m.agents->agents_count : 0;
	if (A != agents_uploaded_)
		upload_agents(m); // agents were added or removed: the whole SoA
	else if (A)
		check(pcg_update_agents(ctx_, m.agents->positions.data(), m.agents->is_active.data()));
}

void gb300_solver::refresh_bulk(microenvironment& m)
{
	if (!m.bulk_fnc)
	{
		check(pcg_set_bulk(ctx_, PCG_BULK_NONE, nullptr, nullptr, nullptr));
		return;
	}
	// planar [s][z][y][x] tables, sampled once (the reference calls the functor
	// three times per voxel and substrate every step, bulk_solver.cpp:12-49)
	const std::size_t V = m.mesh.voxel_count(), S = m.substrates_count;
	std::vector<real_t> sup(V * S), upt(V * S), tgt(V * S);
	for (index_t s = 0; s < S; s++)
		for (index_t z = 0; z < n_[2]; z++)
			for (index_t y = 0; y < n_[1]; y++)
				for (index_t x = 0; x < n_[0]; x++)
				{
					const std::size_t i = s * V + m.mesh.linearize(x, y, z);
					sup[i] = m.bulk_fnc->supply_rates(s, x, y, z);
					upt[i] = m.bulk_fnc->uptake_rates(s, x, y, z);
					tgt[i] = m.bulk_fnc->supply_target_densities(s, x, y, z);
				}
	check(pcg_set_bulk(ctx_, PCG_BULK_PER_VOXEL, sup.data(), upt.data(), tgt.data()));
}

void gb300_solver::initialize(microenvironment& m)
{
	if (initialized_)
		return;
	if (!ctx_)
		check(pcg_create(&ctx_, precision_, device_));
	const cartesian_mesh& g = m.mesh;
	const int64_t mins[3] = { g.bounding_box_mins[0], g.bounding_box_mins[1], g.bounding_box_mins[2] };
	const int64_t maxs[3] = { g.bounding_box_maxs[0], g.bounding_box_maxs[1], g.bounding_box_maxs[2] };
	const uint64_t vox[3] = { g.voxel_shape[0], g.voxel_shape[1], g.voxel_shape[2] };
	check(pcg_set_mesh(ctx_, (int)g.dims, mins, maxs, vox));
	uint64_t grid[3];
	check(pcg_get_grid(ctx_, grid));
	for (int a = 0; a < 3; a++)
		n_[a] = grid[a];
	S_ = m.substrates_count;
	check(pcg_set_substrates(ctx_, m.substrates_count, m.diffusion_timestep, m.diffusion_coefficients.get(),
							 m.decay_rates.get(), m.initial_conditions.get()));
	upload_dirichlet(m);
	refresh_bulk(m);
	upload_agents(m);
	check(pcg_initialize(ctx_));
	host_.assign(g.voxel_count() * m.substrates_count, 0.0);
	check(pcg_get_field(ctx_, host_.data(), PCG_LAYOUT_INTERLEAVED, PCG_DTYPE_F64));
	initialized_ = true;
}

void gb300_solver::solve(microenvironment& m, index_t iterations)
{
	initialize(m);
	check(pcg_solve(ctx_, iterations));
}

real_t gb300_solver::get_substrate_density(index_t s, index_t x, index_t y, index_t z) const
{
	return host_.at(index(s, x, y, z));
}

real_t& gb300_solver::get_substrate_density(index_t s, index_t x, index_t y, index_t z)
{
	return host_.at(index(s, x, y, z));
}

void gb300_solver::transfer_to_device(microenvironment& m)
{
	initialize(m);
	check(pcg_set_field(ctx_, host_.data(), PCG_LAYOUT_INTERLEAVED, PCG_DTYPE_F64));
	refresh_agents(m);
	if (m.agents && m.agents->agents_count)
		check(pcg_set_internalized(ctx_, m.agents->internalized_substrates.data()));
}

void gb300_solver::transfer_to_host(microenvironment& m)
{
	initialize(m);
	check(pcg_get_field(ctx_, host_.data(), PCG_LAYOUT_INTERLEAVED, PCG_DTYPE_F64));
	if (m.agents && m.agents->agents_count)
		check(pcg_get_internalized(ctx_, m.agents->internalized_substrates.data()));
}

void gb300_solver::read_field_planar(real_t* out) const
{
	if (!ctx_)
		throw std::runtime_error("gb300_solver: read before initialize");
	check(pcg_get_field(ctx_, out, PCG_LAYOUT_PLANAR, PCG_DTYPE_F64));
}

void gb300_solver::reinitialize_dirichlet(microenvironment& m)
{
	initialize(m);
	upload_dirichlet(m);
}

void gb300_solver::recompute_positional_data(microenvironment& m)
{
	initialize(m);
	refresh_agents(m);
	check(pcg_recompute_positional_data(ctx_));
}

void gb300_solver::attach_to_registry()
{
	static const registry_adder<gb300_solver> fp64("gb300_solver");
	static const registry_adder<gb300_solver_fp32> fp32("gb300_solver_fp32");
}

} // namespace physicore::biofvm::kernels::gb300_solver
