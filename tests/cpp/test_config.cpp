// Tests of the settings reader, the microenvironment builder and the VTK image
// serializer of the host mirror, after the reference's tests of the same parts
// (reactions-diffusion/biofvm/tests/test_config_reader.cpp,
// test_microenvironment_builder.cpp): parsing of every field, the legacy and
// per-face Dirichlet forms, each required tag missing, malformed XML, and the
// builder's checks.  The serializer writes through a CPU test solver whose
// densities are a known formula; the Python side reads the files back.  No GPU.
//
//   test_config <scratch dir>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <functional>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "../../physicore_gb300/csrc/host/config_reader.h"
#include "../../physicore_gb300/csrc/host/microenvironment.h"
#include "../../physicore_gb300/csrc/host/microenvironment_builder.h"
#include "../../physicore_gb300/csrc/host/solver_registry.h"
#include "../../physicore_gb300/csrc/host/xml_reader.h"

using namespace physicore;
using namespace physicore::biofvm;

static int g_failures = 0;
#define EXPECT(cond)                                                                                         \
	do                                                                                                       \
	{                                                                                                        \
		if (!(cond))                                                                                         \
		{                                                                                                    \
			std::printf("  FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);                                 \
			g_failures++;                                                                                    \
		}                                                                                                    \
	} while (0)
#define EXPECT_NEAR(a, b, tol) EXPECT(std::fabs((double)(a) - (double)(b)) <= (tol))

// Expects `fn` to throw std::runtime_error whose message contains `needle`.
#define EXPECT_THROW_WITH(stmt, needle)                                                                      \
	do                                                                                                       \
	{                                                                                                        \
		bool thrown = false;                                                                                 \
		try                                                                                                  \
		{                                                                                                    \
			stmt;                                                                                            \
		}                                                                                                    \
		catch (const std::runtime_error& e)                                                                  \
		{                                                                                                    \
			thrown = std::string(e.what()).find(needle) != std::string::npos;                                \
			if (!thrown)                                                                                     \
				std::printf("  message was: %s\n", e.what());                                               \
		}                                                                                                    \
		EXPECT(thrown);                                                                                      \
	} while (0)

namespace {

std::string g_scratch;

// Densities s*1000 + x + 10*y + 100*z + 0.25*steps taken.
class formula_solver : public solver
{
public:
	void initialize(microenvironment& m) override
	{
		n_ = m.mesh.grid_shape;
		S_ = m.substrates_count;
		values_.assign(m.mesh.voxel_count() * S_, 0.0);
		fill();
	}
	void solve(microenvironment&, index_t iterations) override
	{
		steps_ += iterations;
		fill();
	}
	real_t get_substrate_density(index_t s, index_t x, index_t y, index_t z) const override
	{
		return values_.at(s + S_ * (x + n_[0] * (y + n_[1] * z)));
	}
	real_t& get_substrate_density(index_t s, index_t x, index_t y, index_t z) override
	{
		return values_.at(s + S_ * (x + n_[0] * (y + n_[1] * z)));
	}
	void reinitialize_dirichlet(microenvironment&) override {}
	void recompute_positional_data(microenvironment&) override {}

private:
	void fill()
	{
		for (index_t z = 0; z < n_[2]; z++)
			for (index_t y = 0; y < n_[1]; y++)
				for (index_t x = 0; x < n_[0]; x++)
					for (index_t s = 0; s < S_; s++)
						get_substrate_density(s, x, y, z) = s * 1000.0 + x + 10.0 * y + 100.0 * z + 0.25 * steps_;
	}
	std::array<index_t, 3> n_ {};
	index_t S_ = 0, steps_ = 0;
	std::vector<real_t> values_;
};

const registry_adder<formula_solver> g_formula("formula_solver");

const char* const kSettings = R"(<?xml version="1.0" encoding="UTF-8"?>
<!-- settings for the reader tests -->
<!DOCTYPE PhysiCell_settings>
<PhysiCell_settings version="devel-version">
    <domain>
        <x_min>-100</x_min> <x_max>60</x_max>
        <y_min>-40</y_min>  <y_max>40</y_max>
        <z_min>0</z_min>    <z_max>40</z_max>
        <dx>20</dx> <dy>20</dy> <dz>20</dz>
        <use_2D>false</use_2D>
    </domain>
    <overall>
        <max_time units="min">2.5</max_time>
        <time_units>min</time_units>
        <space_units>micron</space_units>
        <dt_diffusion units="min">0.05</dt_diffusion>
        <dt_mechanics units="min">0.1</dt_mechanics>
        <dt_phenotype units="min">6</dt_phenotype>
    </overall>
    <microenvironment_setup>
        <variable name="oxygen" units="mmHg" ID="0">
            <physical_parameter_set>
                <diffusion_coefficient units="micron^2/min">1e5</diffusion_coefficient>
                <decay_rate units="1/min">0.1</decay_rate>
            </physical_parameter_set>
            <initial_condition units="mmHg">38.0</initial_condition>
            <Dirichlet_boundary_condition units="mmHg" enabled="True">21.5</Dirichlet_boundary_condition>
            <Dirichlet_options>
                <boundary_value ID="xmax" enabled="False">7.0</boundary_value>
                <boundary_value ID="zmin" enabled="true">3.25</boundary_value>
            </Dirichlet_options>
        </variable>
        <variable name="a &amp; b &#x3b1;" units="&lt;mM&gt;" ID="7">
            <physical_parameter_set>
                <diffusion_coefficient>  600.5 </diffusion_coefficient>
                <decay_rate><![CDATA[0.25]]></decay_rate>
            </physical_parameter_set>
            <initial_condition>15</initial_condition>
            <Dirichlet_boundary_condition enabled="false">99</Dirichlet_boundary_condition>
            <Dirichlet_options>
                <boundary_value ID="ymin" enabled="yes">1.5</boundary_value>
            </Dirichlet_options>
        </variable>
        <options>
            <calculate_gradients>true</calculate_gradients>
            <track_internalized_substrates_in_each_agent>1</track_internalized_substrates_in_each_agent>
        </options>
    </microenvironment_setup>
    <solver><name>formula_solver</name></solver>
</PhysiCell_settings>
)";

std::string replace(std::string s, const std::string& from, const std::string& to)
{
	const std::size_t k = s.find(from);
	if (k == std::string::npos)
		throw std::logic_error("test text does not contain " + from);
	return s.replace(k, from.size(), to);
}

std::string write_file(const std::string& name, const std::string& text)
{
	const std::string path = (std::filesystem::path(g_scratch) / name).string();
	std::ofstream(path, std::ios::binary) << text;
	return path;
}

void parses_every_field()
{
	const physicell_config c = parse_physicell_config(write_file("settings.xml", kSettings));
	EXPECT(c.domain.x_min == -100 && c.domain.x_max == 60 && c.domain.y_min == -40 && c.domain.y_max == 40);
	EXPECT(c.domain.z_min == 0 && c.domain.z_max == 40 && c.domain.dx == 20 && c.domain.dy == 20);
	EXPECT(c.domain.dz == 20 && !c.domain.use_2D);
	EXPECT(c.overall.max_time == 2.5 && c.overall.dt_diffusion == 0.05 && c.overall.dt_mechanics == 0.1);
	EXPECT(c.overall.dt_phenotype == 6 && c.overall.time_units == "min" && c.overall.space_units == "micron");
	EXPECT(c.microenvironment.variables.size() == 2);
	const variable_config& o = c.microenvironment.variables[0];
	EXPECT(o.name == "oxygen" && o.units == "mmHg" && o.id == 0);
	EXPECT(o.diffusion_coefficient == 1e5 && o.decay_rate == 0.1 && o.initial_condition == 38.0);
	// legacy condition on all faces, then xmax switched off and zmin overridden
	const auto& ob = o.boundary_conditions;
	EXPECT(ob.mins_conditions[0] && ob.mins_conditions[1] && ob.mins_conditions[2]);
	EXPECT(!ob.maxs_conditions[0] && ob.maxs_conditions[1] && ob.maxs_conditions[2]);
	EXPECT(ob.mins_values[0] == 21.5 && ob.mins_values[1] == 21.5 && ob.mins_values[2] == 3.25);
	EXPECT(ob.maxs_values[0] == 7.0 && ob.maxs_values[1] == 21.5 && ob.maxs_values[2] == 21.5);
	const variable_config& g = c.microenvironment.variables[1];
	EXPECT(g.name == "a & b \xCE\xB1" && g.units == "<mM>" && g.id == 7);
	EXPECT(g.diffusion_coefficient == 600.5 && g.decay_rate == 0.25 && g.initial_condition == 15);
	// a disabled legacy condition leaves the faces off; ymin set by the options
	const auto& gb = g.boundary_conditions;
	EXPECT(gb.mins_conditions[1] && gb.mins_values[1] == 1.5);
	EXPECT(!gb.mins_conditions[0] && !gb.mins_conditions[2] && gb.mins_values[0] == 0.0);
	EXPECT(!gb.maxs_conditions[0] && !gb.maxs_conditions[1] && !gb.maxs_conditions[2]);
	EXPECT(c.microenvironment.calculate_gradients && c.microenvironment.track_internalized_substrates);
	EXPECT(c.solver.name == "formula_solver");
}

void optional_sections()
{
	std::string t = replace(kSettings, "<solver><name>formula_solver</name></solver>", "");
	const std::size_t a = t.find("<options>"), b = t.find("</options>") + std::strlen("</options>");
	t.erase(a, b - a);
	const physicell_config c = parse_physicell_config_text(t);
	EXPECT(c.solver.name.empty());
	EXPECT(!c.microenvironment.calculate_gradients && !c.microenvironment.track_internalized_substrates);
}

void missing_tags_and_files()
{
	EXPECT_THROW_WITH(parse_physicell_config(std::filesystem::path(g_scratch) / "absent.xml"),
					  "Configuration file not found");
	EXPECT_THROW_WITH(parse_physicell_config_text(replace(kSettings, "<dx>20</dx>", "")),
					  "Required XML tag <dx> not found under <domain>");
	EXPECT_THROW_WITH(parse_physicell_config_text(replace(kSettings, "<time_units>min</time_units>", "")),
					  "Required XML tag <time_units> not found under <overall>");
	EXPECT_THROW_WITH(parse_physicell_config_text(replace(kSettings, "<initial_condition>15</initial_condition>", "")),
					  "Required XML tag <initial_condition> not found under <variable>");
	EXPECT_THROW_WITH(
		parse_physicell_config_text(replace(kSettings, "<decay_rate units=\"1/min\">0.1</decay_rate>", "")),
		"Required XML tag <decay_rate> not found under <physical_parameter_set>");
	std::string no_vars = kSettings;
	const std::size_t a = no_vars.find("<variable name=\"oxygen\""), b = no_vars.find("<options>");
	no_vars.erase(a, b - a);
	EXPECT_THROW_WITH(parse_physicell_config_text(no_vars), "No <variable> tags found");
	EXPECT_THROW_WITH(parse_physicell_config_text(replace(kSettings, "<PhysiCell_settings version=\"devel-version\">",
														  "<Other>")),
					  "Failed to parse XML");
	EXPECT_THROW_WITH(parse_physicell_config_text("<?xml version=\"1.0\"?><Other></Other>"),
					  "Root <PhysiCell_settings> tag not found");
	EXPECT_THROW_WITH(parse_physicell_config_text(replace(kSettings, "</domain>", "")), "Failed to parse XML");
	EXPECT_THROW_WITH(parse_physicell_config_text(replace(kSettings, "&amp;", "&bogus;")), "unknown entity");
}

void xml_reader_forms()
{
	xml::document d;
	std::string err;
	EXPECT(d.parse("<r a='1' b=\"x&quot;y\"><c/><c k=\"2\">t</c><d>u<!-- c -->v</d></r>", err));
	const xml::node* r = d.child("r");
	EXPECT(r && *r->attribute("a") == "1" && *r->attribute("b") == "x\"y");
	EXPECT(r->child("c") && r->child("c")->next_sibling("c") && r->child("c")->next_sibling("c")->text == "t");
	EXPECT(r->find_child_by_attribute("c", "k", "2") == r->child("c")->next_sibling("c"));
	EXPECT(r->child("d")->text == "uv");
	EXPECT(xml::as_bool(std::string(" True")) && !xml::as_bool(std::string("false")) && !xml::as_bool(nullptr));
	EXPECT(xml::as_double(std::string("")) == 0.0 && xml::as_double(std::string(" -2.5e1 ")) == -25.0);
	EXPECT(!d.parse("<a><b></a>", err) && err.find("does not match") != std::string::npos);
	EXPECT(!d.parse("<a></a><b/>", err) && err.find("more than one root") != std::string::npos);
	EXPECT(!d.parse("<a x=1/>", err) && err.find("quoted") != std::string::npos);
	EXPECT(!d.parse("", err) && err.find("no root") != std::string::npos);
}

void create_from_config_builds()
{
	const std::string path = write_file("settings_build.xml", kSettings);
	// create_from_config serialises under ./output: run it from the scratch folder
	const auto cwd = std::filesystem::current_path();
	std::filesystem::current_path(g_scratch);
	std::unique_ptr<microenvironment> m;
	try
	{
		m = microenvironment::create_from_config(path);
	}
	catch (...)
	{
		std::filesystem::current_path(cwd);
		throw;
	}
	std::filesystem::current_path(cwd);
	EXPECT(m->mesh.dims == 3 && m->mesh.grid_shape[0] == 8 && m->mesh.grid_shape[1] == 4 && m->mesh.grid_shape[2] == 2);
	EXPECT(m->diffusion_timestep == 0.05 && m->simulation_time == 2.5 && m->time_units == "min");
	EXPECT(m->substrates_count == 2 && m->substrates_names[1] == "a & b \xCE\xB1");
	EXPECT(m->diffusion_coefficients[0] == 1e5 && m->decay_rates[1] == 0.25 && m->initial_conditions[1] == 15);
	EXPECT(m->compute_internalized_substrates);
	EXPECT(m->agents && m->agents->agents_count == 0 && m->agents->dims == 3 && m->agents->substrate_count == 2);
	EXPECT(m->dirichlet_interior_voxels_count == 0);
	// every face is used by oxygen except x-max, which no density uses
	EXPECT(m->dirichlet_min_boundary_values[0] && m->dirichlet_min_boundary_values[1] &&
		   m->dirichlet_min_boundary_values[2]);
	EXPECT(!m->dirichlet_max_boundary_values[0] && !m->dirichlet_max_boundary_conditions[0]);
	EXPECT(m->dirichlet_max_boundary_values[1] && m->dirichlet_max_boundary_values[2]);
	EXPECT(m->dirichlet_min_boundary_conditions[1][0] && m->dirichlet_min_boundary_conditions[1][1]);
	EXPECT(m->dirichlet_min_boundary_values[1][1] == 1.5 && m->dirichlet_min_boundary_values[2][0] == 3.25);
	EXPECT(!m->dirichlet_max_boundary_conditions[1][1] && m->dirichlet_max_boundary_values[1][0] == 21.5);
	EXPECT(m->serializer != nullptr);
	EXPECT(std::filesystem::is_directory(std::filesystem::path(g_scratch) / "output" / "vtk_microenvironment"));
	// 2-D: the z faces are dropped and the mesh has one z layer
	std::string t2 = replace(kSettings, "<use_2D>false</use_2D>", "<use_2D>true</use_2D>");
	t2 = replace(t2, "<dz>20</dz>", "<dz>0</dz>");
	microenvironment_builder b;
	configure_from(b, parse_physicell_config_text(t2));
	b.set_output_dir("");
	const auto m2 = b.build();
	EXPECT(m2->mesh.dims == 2 && m2->mesh.grid_shape[2] == 1 && !m2->dirichlet_min_boundary_values[2]);
	EXPECT(m2->serializer == nullptr);
	// negative voxel edges are rejected before the mesh is made
	EXPECT_THROW_WITH(configure_from(b, parse_physicell_config_text(replace(kSettings, "<dy>20</dy>", "<dy>-1</dy>"))),
					  "Voxel dimensions must be positive");
}

void builder_checks()
{
	{
		microenvironment_builder b;
		b.add_density("x", "u", 1, 1, 1);
		EXPECT_THROW_WITH(b.build(), "without a mesh");
		EXPECT_THROW_WITH(b.add_dirichlet_node({ 0, 0, 0 }, { 1.0 }), "without a mesh");
	}
	{
		microenvironment_builder b;
		b.resize(2, { 0, 0, 0 }, { 100, 100, 0 }, { 20, 20, 20 });
		EXPECT_THROW_WITH(b.build(), "no densities");
		b.add_density("a", "u", 1, 0.5, 2);
		b.add_density("b", "u", 3, 0.25, 4);
		EXPECT(b.get_density_index("b") == 1);
		EXPECT_THROW_WITH(b.get_density_index("c"), "Density c not found");
		EXPECT_THROW_WITH(b.add_dirichlet_node({ 1, 1, 0 }, { 1.0 }), "values size");
		EXPECT_THROW_WITH(b.add_dirichlet_node({ 1, 1, 0 }, { 1.0, 2.0 }, { true }), "conditions size");
		EXPECT_THROW_WITH(b.add_boundary_dirichlet_conditions(2, {}, {}, {}, {}), "out of bounds");
		b.add_dirichlet_node({ 1, 2, 9 }, { 5.0, 6.0 });
		b.add_dirichlet_node({ 3, 4, 9 }, { 7.0, 8.0 }, { false, true });
		b.select_solver("no_such_solver");
		b.set_output_dir("");
		EXPECT_THROW_WITH(b.build(), "Can not find solver for microenvironment: no_such_solver");
		b.select_solver("formula_solver");
		const auto m = b.build();
		EXPECT(m->dirichlet_interior_voxels_count == 2);
		EXPECT(m->dirichlet_interior_voxels[0] == 1 && m->dirichlet_interior_voxels[1] == 2 &&
			   m->dirichlet_interior_voxels[2] == 3 && m->dirichlet_interior_voxels[3] == 4);
		EXPECT(m->dirichlet_interior_values[3] == 8.0 && m->dirichlet_interior_conditions[0] &&
			   m->dirichlet_interior_conditions[1] && !m->dirichlet_interior_conditions[2]);
		EXPECT(!m->dirichlet_min_boundary_values[0] && !m->dirichlet_max_boundary_values[1]);
	}
}

// Writes two images of a 3-D and one of a 2-D microenvironment through the
// formula solver; the Python test checks the files' contents.
void serializer_writes()
{
	for (int dims : { 3, 2 })
	{
		microenvironment_builder b;
		b.resize(dims, { -40, 20, -60 }, { 60, 80, 0 }, { 20, 20, 30 });
		b.add_density("first", "u", 1, 0, 0);
		b.add_density("second one", "u", 1, 0, 0);
		b.add_density("third", "u", 1, 0, 0);
		b.select_solver("formula_solver");
		b.set_simulation_time(1.0);
		b.set_output_dir((std::filesystem::path(g_scratch) / ("out" + std::to_string(dims))).string());
		const auto m = b.build();
		m->solver->initialize(*m);
		m->serialize_state(0.0);
		m->run_single_timestep();
		m->run_single_timestep();
		m->serialize_state(0.125);
	}
	EXPECT(std::filesystem::exists(std::filesystem::path(g_scratch) / "out3" / "vtk_microenvironment" /
								   "microenvironment_000001.vti"));
	EXPECT(std::filesystem::exists(std::filesystem::path(g_scratch) / "out2" / "microenvironment.pvd"));
}

// Corrupted settings (random deletions, insertions and replacements of
// characters) either parse or throw std::runtime_error: the reader never crashes,
// hangs or throws anything else.
void mutated_settings_fail_cleanly()
{
	std::mt19937_64 rng(12345);
	const std::string base = kSettings;
	const char alphabet[] = "<>/=\"'&;!?-[]abcxyz0129 \n";
	int parsed = 0, rejected = 0;
	for (int trial = 0; trial < 3000; trial++)
	{
		std::string t = base;
		const int edits = 1 + (int)(rng() % 6);
		for (int e = 0; e < edits && !t.empty(); e++)
		{
			const std::size_t at = rng() % t.size();
			const char ch = alphabet[rng() % (sizeof alphabet - 1)];
			switch (rng() % 3)
			{
			case 0: t.erase(at, 1 + rng() % 8); break;
			case 1: t.insert(at, 1, ch); break;
			default: t[at] = ch; break;
			}
		}
		try
		{
			(void)parse_physicell_config_text(t);
			parsed++;
		}
		catch (const std::runtime_error&)
		{
			rejected++;
		}
	}
	EXPECT(parsed + rejected == 3000 && rejected > 0);
}

struct test_case
{
	const char* name;
	std::function<void()> fn;
};

} // namespace

int main(int argc, char** argv)
{
	if (argc < 2)
	{
		std::printf("usage: test_config <scratch dir>\n");
		return 2;
	}
	g_scratch = argv[1];
	std::filesystem::create_directories(g_scratch);
	const test_case tests[] = {
		{ "ConfigReaderTest.ParsesEveryField", parses_every_field },
		{ "ConfigReaderTest.OptionalSections", optional_sections },
		{ "ConfigReaderTest.MissingTagsAndFiles", missing_tags_and_files },
		{ "XmlReaderTest.Forms", xml_reader_forms },
		{ "MicroenvironmentTest.CreateFromConfig", create_from_config_builds },
		{ "MicroenvironmentBuilderTest.Checks", builder_checks },
		{ "VtkSerializerTest.Writes", serializer_writes },
		{ "ConfigReaderTest.MutatedSettingsFailCleanly", mutated_settings_fail_cleanly },
	};
	int ran = 0;
	for (const auto& t : tests)
	{
		const int before = g_failures;
		try
		{
			t.fn();
		}
		catch (const std::exception& e)
		{
			std::printf("  EXCEPTION: %s\n", e.what());
			g_failures++;
		}
		std::printf("[%s] %s\n", g_failures == before ? "  OK  " : "FAILED", t.name);
		ran++;
	}
	std::printf("%d tests, %d failures\n", ran, g_failures);
	return g_failures ? 1 : 0;
}
