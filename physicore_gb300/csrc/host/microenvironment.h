// microenvironment.h -- the problem a solver reads, with the reference's field
// names (reactions-diffusion/biofvm/include/biofvm/microenvironment.h:46-81): mesh,
// substrates, Dirichlet interior voxels and boundary faces, bulk functor, agents.
#pragma once

#include <array>
#include <memory>
#include <stdexcept>

#include "agent_data.h"
#include "bulk_functor.h"
#include "mesh.h"
#include "solver.h"
#include "types.h"

namespace physicore::biofvm {

struct microenvironment
{
	microenvironment(const cartesian_mesh& mesh, index_t substrates_count, real_t timestep)
		: diffusion_timestep(timestep), mesh(mesh), substrates_count(substrates_count),
		  initial_conditions(std::make_unique<real_t[]>(substrates_count)),
		  diffusion_coefficients(std::make_unique<real_t[]>(substrates_count)),
		  decay_rates(std::make_unique<real_t[]>(substrates_count))
	{}

	microenvironment(const microenvironment&) = delete;
	microenvironment& operator=(const microenvironment&) = delete;

	// One step of the solver (microenvironment::run_single_timestep,
	// src/microenvironment.cpp:87)
	void run_single_timestep()
	{
		if (!solver)
			throw std::runtime_error("no solver selected");
		solver->solve(*this, 1);
	}

	std::unique_ptr<agent_data> agents;
	solver_ptr solver;

	real_t diffusion_timestep;
	cartesian_mesh mesh;

	index_t substrates_count;
	std::unique_ptr<real_t[]> initial_conditions;
	std::unique_ptr<real_t[]> diffusion_coefficients;
	std::unique_ptr<real_t[]> decay_rates;

	index_t dirichlet_interior_voxels_count = 0;
	std::unique_ptr<index_t[]> dirichlet_interior_voxels; // count * dims
	std::unique_ptr<real_t[]> dirichlet_interior_values;  // count * substrates
	std::unique_ptr<bool[]> dirichlet_interior_conditions;

	std::array<std::unique_ptr<real_t[]>, 3> dirichlet_min_boundary_values = { nullptr, nullptr, nullptr };
	std::array<std::unique_ptr<real_t[]>, 3> dirichlet_max_boundary_values = { nullptr, nullptr, nullptr };
	std::array<std::unique_ptr<bool[]>, 3> dirichlet_min_boundary_conditions = { nullptr, nullptr, nullptr };
	std::array<std::unique_ptr<bool[]>, 3> dirichlet_max_boundary_conditions = { nullptr, nullptr, nullptr };

	std::unique_ptr<bulk_functor> bulk_fnc;

	bool compute_internalized_substrates = false;
};

} // namespace physicore::biofvm
