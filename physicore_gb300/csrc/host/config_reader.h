// config_reader.h -- PhysiCell_settings.xml into plain structures, with the
// reference's structure and field names (reactions-diffusion/biofvm/src/
// config_reader.h:10-80) and its behaviour (src/config_reader.cpp:1-258):
//   * the file must exist and parse, and its root must be <PhysiCell_settings>;
//   * <domain>, <overall> and <microenvironment_setup> are required, with every
//     child tag the reference reads (a missing one throws std::runtime_error naming
//     the tag and its parent); at least one <variable> is required;
//   * per variable, a legacy <Dirichlet_boundary_condition enabled=...> sets all six
//     faces, and <Dirichlet_options>/<boundary_value ID="xmin".."zmax"> entries then
//     override single faces;
//   * <options> and <solver> are optional (false / empty name when absent).
// Domain validation is left to the builder, as in the reference.
#pragma once

#include <array>
#include <filesystem>
#include <string>
#include <vector>

#include "types.h"

namespace physicore {

struct domain_config
{
	real_t x_min;
	real_t x_max;
	real_t y_min;
	real_t y_max;
	real_t z_min;
	real_t z_max;
	real_t dx;
	real_t dy;
	real_t dz;
	bool use_2D;
};

struct overall_config
{
	real_t max_time;
	std::string time_units;
	std::string space_units;
	real_t dt_diffusion;
	real_t dt_mechanics;
	real_t dt_phenotype;
};

struct dirichlet_boundary_config
{
	std::array<real_t, 3> mins_values;	 // x, y, z
	std::array<real_t, 3> maxs_values;	 // x, y, z
	std::array<bool, 3> mins_conditions; // enabled flags
	std::array<bool, 3> maxs_conditions;
};

struct variable_config
{
	std::string name;
	std::string units;
	index_t id;
	real_t diffusion_coefficient;
	real_t decay_rate;
	real_t initial_condition;
	dirichlet_boundary_config boundary_conditions;
};

struct solver_config
{
	std::string name;
};

struct microenvironment_config
{
	std::vector<variable_config> variables;
	bool calculate_gradients;
	bool track_internalized_substrates;
};

struct physicell_config
{
	domain_config domain;
	overall_config overall;
	microenvironment_config microenvironment;
	solver_config solver;
};

// Parses a settings file; throws std::runtime_error on a missing file, malformed
// XML or a missing required tag.
physicell_config parse_physicell_config(const std::filesystem::path& config_file);

// The same from XML text (`origin` names it in error messages).
physicell_config parse_physicell_config_text(const std::string& text, const std::string& origin = "<text>");

} // namespace physicore
