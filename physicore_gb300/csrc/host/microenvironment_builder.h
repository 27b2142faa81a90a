// microenvironment_builder.h -- step-by-step construction of a microenvironment,
// with the reference's methods and checks (reactions-diffusion/biofvm/include/
// biofvm/microenvironment_builder.h, src/microenvironment_builder.cpp:14-212):
//   * build() needs a mesh and at least one density, and a registered solver name
//     (std::runtime_error otherwise);
//   * face conditions become per-axis arrays only for the axes (below the mesh's
//     dims) where some density uses that face;
//   * Dirichlet nodes take one value per density and optional conditions (all
//     true when omitted);
//   * the built microenvironment gets agent storage for its dims and densities and
//     a VTK image serializer writing under the output directory ("output" as in
//     the reference; an empty directory attaches none).
#pragma once

#include <array>
#include <memory>
#include <optional>
#include <string>
#include <string_view>
#include <vector>

#include "bulk_functor.h"
#include "config_reader.h"
#include "mesh.h"
#include "microenvironment.h"
#include "types.h"

namespace physicore::biofvm {

class microenvironment_builder
{
public:
	void set_name(std::string_view name);
	void set_time_units(std::string_view time_units);
	void set_space_units(std::string_view space_units);
	void set_time_step(real_t time_step);
	void set_simulation_time(real_t simulation_time);

	void resize(index_t dims, std::array<sindex_t, 3> bounding_box_mins, std::array<sindex_t, 3> bounding_box_maxs,
				std::array<index_t, 3> voxel_shape);

	void add_density(const std::string& name, const std::string& units, real_t diffusion_coefficient,
					 real_t decay_rate, real_t initial_condition);
	std::size_t get_density_index(const std::string& name) const;

	void add_dirichlet_node(std::array<index_t, 3> voxel_index, std::vector<real_t> values,
							std::vector<bool> conditions = {});
	void add_boundary_dirichlet_conditions(std::size_t density_index, std::array<real_t, 3> mins_values,
										   std::array<real_t, 3> maxs_values, std::array<bool, 3> mins_conditions,
										   std::array<bool, 3> maxs_conditions);

	void set_bulk_functions(std::unique_ptr<bulk_functor> functor);
	void do_compute_internalized_substrates();
	void select_solver(const std::string& name);

	// Where build() points the serializer ("output" by default; empty: none).
	void set_output_dir(std::string_view dir);

	std::unique_ptr<microenvironment> build();

private:
	void fill_dirichlet_vectors(microenvironment& m) const;

	std::string name, time_units, space_units;
	real_t timestep = 0, simulation_time = 0;
	std::optional<cartesian_mesh> mesh;

	std::vector<std::string> substrates_names, substrates_units;
	std::vector<real_t> diffusion_coefficients, decay_rates, initial_conditions;

	std::vector<index_t> dirichlet_voxels;
	std::vector<real_t> dirichlet_values;
	std::vector<bool> dirichlet_conditions;

	std::vector<std::array<real_t, 3>> boundary_mins_values, boundary_maxs_values;
	std::vector<std::array<bool, 3>> boundary_mins_conditions, boundary_maxs_conditions;

	std::unique_ptr<bulk_functor> bulk_fnc;
	bool compute_internalized_substrates = false;
	std::string solver_name;
	std::string output_dir = "output";
};

// Applies a parsed settings file to a builder, as microenvironment::
// create_from_config does before building (src/microenvironment.cpp:22-85): run
// metadata, mesh (bounds and voxel edges truncated to integers, 2-D when use_2D,
// voxel edges must be positive), densities with their face conditions,
// internalized tracking and the solver name when given.
void configure_from(microenvironment_builder& b, const physicell_config& config);

} // namespace physicore::biofvm
