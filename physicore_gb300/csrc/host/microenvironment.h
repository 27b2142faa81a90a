// microenvironment.h -- the problem a solver reads, with the reference's field
// names (reactions-diffusion/biofvm/include/biofvm/microenvironment.h:46-81): mesh,
// substrates, Dirichlet interior voxels and boundary faces, bulk functor, agents,
// the run's metadata and its serializer; create_from_config builds one from a
// PhysiCell_settings.xml file as src/microenvironment.cpp:22-85 does.
#pragma once

#include <array>
#include <filesystem>
#include <iosfwd>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "agent_data.h"
#include "bulk_functor.h"
#include "mesh.h"
#include "serializer.h"
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

	// Reads a settings file and builds through microenvironment_builder: mesh from
	// <domain> (bounds truncated to integers, 2-D when use_2D), one density per
	// <variable> with its face conditions, internalized tracking from <options>,
	// the solver named by <solver> (throws std::runtime_error on any error).
	static std::unique_ptr<microenvironment> create_from_config(const std::filesystem::path& config_file);

	// One step of the solver (microenvironment::run_single_timestep,
	// src/microenvironment.cpp:87)
	void run_single_timestep()
	{
		if (!solver)
			throw std::runtime_error("no solver selected");
		solver->solve(*this, 1);
	}

	// Writes the state through the attached serializer, if any.
	void serialize_state(real_t current_time);

	real_t get_substrate_density(index_t s, index_t x, index_t y, index_t z) const
	{
		return static_cast<const biofvm::solver&>(*solver).get_substrate_density(s, x, y, z);
	}

	// The configuration summary of src/microenvironment.cpp:103-136.
	void print_info(std::ostream& os) const;

	std::string name;
	std::string time_units;
	std::string space_units;
	real_t simulation_time = 0;

	std::unique_ptr<agent_data> agents;
	solver_ptr solver;
	std::unique_ptr<biofvm::serializer> serializer;

	real_t diffusion_timestep;
	cartesian_mesh mesh;

	index_t substrates_count;
	std::vector<std::string> substrates_names;
	std::vector<std::string> substrates_units;
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
