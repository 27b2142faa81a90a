// microenvironment_builder.cpp -- see microenvironment_builder.h; also the
// microenvironment members that need the builder, the config reader or a
// serializer (create_from_config, serialize_state, print_info).
#include "microenvironment_builder.h"

#include <algorithm>
#include <ostream>
#include <stdexcept>

#include "config_reader.h"
#include "solver_registry.h"
#include "vtk_serializer.h"

namespace physicore::biofvm {

void microenvironment_builder::set_name(std::string_view v) { name = v; }
void microenvironment_builder::set_time_units(std::string_view v) { time_units = v; }
void microenvironment_builder::set_space_units(std::string_view v) { space_units = v; }
void microenvironment_builder::set_time_step(real_t v) { timestep = v; }
void microenvironment_builder::set_simulation_time(real_t v) { simulation_time = v; }
void microenvironment_builder::set_output_dir(std::string_view dir) { output_dir = dir; }

void microenvironment_builder::resize(index_t dims, std::array<sindex_t, 3> mins, std::array<sindex_t, 3> maxs,
									  std::array<index_t, 3> voxel_shape)
{
	mesh.emplace(dims, mins, maxs, voxel_shape);
}

void microenvironment_builder::add_density(const std::string& density_name, const std::string& units,
										   real_t diffusion_coefficient, real_t decay_rate, real_t initial_condition)
{
	substrates_names.push_back(density_name);
	substrates_units.push_back(units);
	diffusion_coefficients.push_back(diffusion_coefficient);
	decay_rates.push_back(decay_rate);
	initial_conditions.push_back(initial_condition);
	boundary_mins_values.push_back({ 0, 0, 0 });
	boundary_maxs_values.push_back({ 0, 0, 0 });
	boundary_mins_conditions.push_back({ false, false, false });
	boundary_maxs_conditions.push_back({ false, false, false });
}

std::size_t microenvironment_builder::get_density_index(const std::string& density_name) const
{
	const auto it = std::find(substrates_names.begin(), substrates_names.end(), density_name);
	if (it == substrates_names.end())
		throw std::runtime_error("Density " + density_name + " not found");
	return (std::size_t)(it - substrates_names.begin());
}

void microenvironment_builder::add_dirichlet_node(std::array<index_t, 3> voxel_index, std::vector<real_t> values,
												  std::vector<bool> conditions)
{
	const std::size_t S = substrates_names.size();
	if (values.size() != S)
		throw std::runtime_error("Dirichlet node values size does not match the number of densities");
	if (!conditions.empty() && conditions.size() != S)
		throw std::runtime_error("Dirichlet node conditions size does not match the number of densities");
	if (!mesh)
		throw std::runtime_error("Dirichlet node cannot be added without a mesh");
	for (index_t a = 0; a < mesh->dims; a++)
		dirichlet_voxels.push_back(voxel_index[a]);
	dirichlet_values.insert(dirichlet_values.end(), values.begin(), values.end());
	if (conditions.empty())
		conditions.assign(S, true);
	dirichlet_conditions.insert(dirichlet_conditions.end(), conditions.begin(), conditions.end());
}

void microenvironment_builder::add_boundary_dirichlet_conditions(std::size_t density_index,
																 std::array<real_t, 3> mins_values,
																 std::array<real_t, 3> maxs_values,
																 std::array<bool, 3> mins_conditions,
																 std::array<bool, 3> maxs_conditions)
{
	if (density_index >= substrates_names.size())
		throw std::runtime_error("Density index out of bounds");
	boundary_mins_values[density_index] = mins_values;
	boundary_maxs_values[density_index] = maxs_values;
	boundary_mins_conditions[density_index] = mins_conditions;
	boundary_maxs_conditions[density_index] = maxs_conditions;
}

void microenvironment_builder::set_bulk_functions(std::unique_ptr<bulk_functor> functor)
{
	bulk_fnc = std::move(functor);
}

void microenvironment_builder::do_compute_internalized_substrates() { compute_internalized_substrates = true; }

void microenvironment_builder::select_solver(const std::string& v) { solver_name = v; }

void microenvironment_builder::fill_dirichlet_vectors(microenvironment& m) const
{
	const index_t S = m.substrates_count;
	auto one_side = [&](index_t axis, const std::vector<std::array<real_t, 3>>& values,
						const std::vector<std::array<bool, 3>>& conditions, std::unique_ptr<real_t[]>& out_values,
						std::unique_ptr<bool[]>& out_conditions) {
		bool used = false;
		for (index_t s = 0; s < S; s++)
			used = used || conditions[s][axis];
		if (!used)
			return; // the face keeps no arrays: the solver skips it
		out_values = std::make_unique<real_t[]>(S);
		out_conditions = std::make_unique<bool[]>(S);
		for (index_t s = 0; s < S; s++)
		{
			out_values[s] = values[s][axis];
			out_conditions[s] = conditions[s][axis];
		}
	};
	for (index_t a = 0; a < m.mesh.dims; a++)
	{
		one_side(a, boundary_mins_values, boundary_mins_conditions, m.dirichlet_min_boundary_values[a],
				 m.dirichlet_min_boundary_conditions[a]);
		one_side(a, boundary_maxs_values, boundary_maxs_conditions, m.dirichlet_max_boundary_values[a],
				 m.dirichlet_max_boundary_conditions[a]);
	}
}

std::unique_ptr<microenvironment> microenvironment_builder::build()
{
	if (!mesh)
		throw std::runtime_error("Microenvironment cannot be built without a mesh");
	if (substrates_names.empty())
		throw std::runtime_error("Microenvironment cannot be built with no densities");
	const index_t S = substrates_names.size();
	auto m = std::make_unique<microenvironment>(*mesh, S, timestep);
	m->name = name;
	m->time_units = time_units;
	m->space_units = space_units;
	m->simulation_time = simulation_time;
	m->substrates_names = substrates_names;
	m->substrates_units = substrates_units;
	std::copy(initial_conditions.begin(), initial_conditions.end(), m->initial_conditions.get());
	std::copy(diffusion_coefficients.begin(), diffusion_coefficients.end(), m->diffusion_coefficients.get());
	std::copy(decay_rates.begin(), decay_rates.end(), m->decay_rates.get());

	m->dirichlet_interior_voxels_count = dirichlet_voxels.size() / m->mesh.dims;
	m->dirichlet_interior_voxels = std::make_unique<index_t[]>(dirichlet_voxels.size());
	std::copy(dirichlet_voxels.begin(), dirichlet_voxels.end(), m->dirichlet_interior_voxels.get());
	m->dirichlet_interior_values = std::make_unique<real_t[]>(dirichlet_values.size());
	std::copy(dirichlet_values.begin(), dirichlet_values.end(), m->dirichlet_interior_values.get());
	m->dirichlet_interior_conditions = std::make_unique<bool[]>(dirichlet_conditions.size());
	std::copy(dirichlet_conditions.begin(), dirichlet_conditions.end(), m->dirichlet_interior_conditions.get());
	fill_dirichlet_vectors(*m);

	m->bulk_fnc = std::move(bulk_fnc);
	m->compute_internalized_substrates = compute_internalized_substrates;
	m->agents = std::make_unique<agent_data>(m->mesh.dims, S);

	m->solver = solver_registry::instance().get(solver_name);
	if (!m->solver)
		throw std::runtime_error("Can not find solver for microenvironment: " + solver_name);
	if (!output_dir.empty())
		m->serializer = std::make_unique<vtk_serializer>(output_dir, *m);
	return m;
}

void configure_from(microenvironment_builder& b, const physicell_config& config)
{
	b.set_name("microenvironment");
	b.set_time_units(config.overall.time_units);
	b.set_space_units(config.overall.space_units);
	b.set_time_step(config.overall.dt_diffusion);
	b.set_simulation_time(config.overall.max_time);

	const domain_config& d = config.domain;
	const index_t dims = d.use_2D ? 2 : 3;
	if (d.dx <= 0 || d.dy <= 0 || (!d.use_2D && d.dz <= 0))
		throw std::runtime_error("Voxel dimensions must be positive");
	// bounds and voxel edges are integers in the mesh: truncated, as the reference casts
	b.resize(dims, { (sindex_t)d.x_min, (sindex_t)d.y_min, (sindex_t)d.z_min },
			 { (sindex_t)d.x_max, (sindex_t)d.y_max, (sindex_t)d.z_max },
			 { (index_t)d.dx, (index_t)d.dy, (index_t)d.dz });

	for (const variable_config& v : config.microenvironment.variables)
	{
		b.add_density(v.name, v.units, v.diffusion_coefficient, v.decay_rate, v.initial_condition);
		const dirichlet_boundary_config& bc = v.boundary_conditions;
		b.add_boundary_dirichlet_conditions(b.get_density_index(v.name), bc.mins_values, bc.maxs_values,
											bc.mins_conditions, bc.maxs_conditions);
	}
	if (config.microenvironment.track_internalized_substrates)
		b.do_compute_internalized_substrates();
	if (!config.solver.name.empty())
		b.select_solver(config.solver.name);
}

std::unique_ptr<microenvironment> microenvironment::create_from_config(const std::filesystem::path& config_file)
{
	microenvironment_builder b;
	configure_from(b, parse_physicell_config(config_file));
	return b.build();
}

void microenvironment::serialize_state(real_t current_time)
{
	if (serializer)
		serializer->serialize(*this, current_time);
}

void microenvironment::print_info(std::ostream& os) const
{
	os << "Microenvironment config:\n";
	os << "  Time units: " << time_units << "\n";
	os << "  Space units: " << space_units << "\n";
	os << "  Timestep: " << diffusion_timestep << " " << time_units << "\n";
	os << "  Dimensions: " << mesh.dims << "D\n";
	os << "  Grid bounds:";
	for (index_t a = 0; a < mesh.dims; a++)
		os << (a ? " x [" : " [") << mesh.bounding_box_mins[a] << ", " << mesh.bounding_box_maxs[a] << "]";
	os << " " << space_units << "\n";
	os << "  Voxel size:";
	for (index_t a = 0; a < mesh.dims; a++)
		os << (a ? " x " : " ") << mesh.voxel_shape[a];
	os << " " << space_units << "\n";
	os << "  Grid shape:";
	for (index_t a = 0; a < mesh.dims; a++)
		os << (a ? " x " : " ") << mesh.grid_shape[a];
	os << "\n  Substrates (" << substrates_count << "):\n";
	for (index_t s = 0; s < substrates_count; s++)
		os << "    " << (s < substrates_names.size() ? substrates_names[s] : std::string("?")) << " ["
		   << (s < substrates_units.size() ? substrates_units[s] : std::string()) << "]: D=" << diffusion_coefficients[s]
		   << ", decay=" << decay_rates[s] << ", initial=" << initial_conditions[s] << "\n";
	os << "  Track internalized substrates: " << (compute_internalized_substrates ? "yes" : "no") << "\n";
	os.flush();
}

} // namespace physicore::biofvm
