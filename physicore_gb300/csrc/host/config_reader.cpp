// config_reader.cpp -- see config_reader.h.
#include "config_reader.h"

#include <fstream>
#include <sstream>
#include <stdexcept>

#include "xml_reader.h"

namespace physicore {

namespace {

using xml::node;

const node& required(const node& parent, const char* name)
{
	const node* c = parent.child(name);
	if (!c)
		throw std::runtime_error(std::string("Required XML tag <") + name + "> not found under <" + parent.name +
								 ">");
	return *c;
}

real_t real_of(const node& parent, const char* name) { return xml::as_double(required(parent, name).text); }
bool bool_of(const node& parent, const char* name) { return xml::as_bool(required(parent, name).text); }

std::string string_of(const node& parent, const char* name)
{
	// pugixml's text() is the first character-data child: surrounding white space kept
	return required(parent, name).text;
}

domain_config read_domain(const node& n)
{
	domain_config d {};
	d.x_min = real_of(n, "x_min");
	d.x_max = real_of(n, "x_max");
	d.y_min = real_of(n, "y_min");
	d.y_max = real_of(n, "y_max");
	d.z_min = real_of(n, "z_min");
	d.z_max = real_of(n, "z_max");
	d.dx = real_of(n, "dx");
	d.dy = real_of(n, "dy");
	d.dz = real_of(n, "dz");
	d.use_2D = bool_of(n, "use_2D");
	return d;
}

overall_config read_overall(const node& n)
{
	overall_config o {};
	o.max_time = real_of(n, "max_time");
	o.time_units = string_of(n, "time_units");
	o.space_units = string_of(n, "space_units");
	o.dt_diffusion = real_of(n, "dt_diffusion");
	o.dt_mechanics = real_of(n, "dt_mechanics");
	o.dt_phenotype = real_of(n, "dt_phenotype");
	return o;
}

dirichlet_boundary_config read_dirichlet(const node& var)
{
	dirichlet_boundary_config b {};
	b.mins_values.fill(0.0);
	b.maxs_values.fill(0.0);
	b.mins_conditions.fill(false);
	b.maxs_conditions.fill(false);
	// the legacy single condition applies to every face when enabled
	if (const node* legacy = var.child("Dirichlet_boundary_condition"))
		if (xml::as_bool(legacy->attribute("enabled")))
		{
			const real_t v = xml::as_double(legacy->text);
			b.mins_values.fill(v);
			b.maxs_values.fill(v);
			b.mins_conditions.fill(true);
			b.maxs_conditions.fill(true);
		}
	const node* options = var.child("Dirichlet_options");
	if (!options)
		return b;
	static const char* const ids[6] = { "xmin", "xmax", "ymin", "ymax", "zmin", "zmax" };
	for (int f = 0; f < 6; f++)
	{
		const node* bv = options->find_child_by_attribute("boundary_value", "ID", ids[f]);
		if (!bv)
			continue;
		const int axis = f / 2;
		const real_t v = xml::as_double(bv->text);
		const bool on = xml::as_bool(bv->attribute("enabled"));
		(f % 2 ? b.maxs_values : b.mins_values)[axis] = v;
		(f % 2 ? b.maxs_conditions : b.mins_conditions)[axis] = on;
	}
	return b;
}

variable_config read_variable(const node& n)
{
	variable_config v {};
	const std::string* name = n.attribute("name");
	const std::string* units = n.attribute("units");
	v.name = name ? *name : std::string();
	v.units = units ? *units : std::string();
	v.id = (index_t)xml::as_uint(n.attribute("ID"));
	const node& params = required(n, "physical_parameter_set");
	v.diffusion_coefficient = real_of(params, "diffusion_coefficient");
	v.decay_rate = real_of(params, "decay_rate");
	v.initial_condition = real_of(n, "initial_condition");
	v.boundary_conditions = read_dirichlet(n);
	return v;
}

microenvironment_config read_microenvironment(const node& n)
{
	microenvironment_config m {};
	for (const node* v = n.child("variable"); v; v = v->next_sibling("variable"))
		m.variables.push_back(read_variable(*v));
	if (m.variables.empty())
		throw std::runtime_error("No <variable> tags found in <microenvironment_setup>");
	m.calculate_gradients = false;
	m.track_internalized_substrates = false;
	if (const node* options = n.child("options"))
	{
		if (const node* g = options->child("calculate_gradients"))
			m.calculate_gradients = xml::as_bool(g->text);
		if (const node* t = options->child("track_internalized_substrates_in_each_agent"))
			m.track_internalized_substrates = xml::as_bool(t->text);
	}
	return m;
}

physicell_config read_document(const xml::document& doc, const std::string& origin)
{
	const node* root = doc.child("PhysiCell_settings");
	if (!root)
		throw std::runtime_error("Root <PhysiCell_settings> tag not found in " + origin);
	physicell_config c {};
	c.domain = read_domain(required(*root, "domain"));
	c.overall = read_overall(required(*root, "overall"));
	c.microenvironment = read_microenvironment(required(*root, "microenvironment_setup"));
	if (const node* s = root->child("solver"))
		c.solver.name = string_of(*s, "name");
	return c;
}

} // namespace

physicell_config parse_physicell_config_text(const std::string& text, const std::string& origin)
{
	xml::document doc;
	std::string error;
	if (!doc.parse(text, error))
		throw std::runtime_error("Failed to parse XML file: " + origin + " - " + error);
	return read_document(doc, origin);
}

physicell_config parse_physicell_config(const std::filesystem::path& config_file)
{
	if (!std::filesystem::exists(config_file))
		throw std::runtime_error("Configuration file not found: " + config_file.string());
	std::ifstream f(config_file, std::ios::binary);
	if (!f)
		throw std::runtime_error("Failed to parse XML file: " + config_file.string() + " - cannot open file");
	std::ostringstream ss;
	ss << f.rdbuf();
	return parse_physicell_config_text(ss.str(), config_file.string());
}

} // namespace physicore
