// Tests of the C++ host mirror of the solver plugin surface and of the gb300_solver
// plugin behind it.  Layout and names follow the reference's gtests
// (reactions-diffusion/biofvm/tests/test_solver_registry.cpp,
// kernels/openmp_solver/tests/test_diffusion_solver.cpp:61-134,
// tests/test_dirichlet_modification.cpp), with a minimal check macro instead of
// gtest.  Run with --cpu for the tests that need no GPU.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <string>
#include <vector>

#include "../../physicore_gb300/csrc/host/gb300_solver.h"
#include "../../physicore_gb300/csrc/host/microenvironment.h"
#include "../../physicore_gb300/csrc/host/solver_registry.h"

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

namespace {

class mock_solver : public solver
{
public:
	void initialize(microenvironment&) override {}
	void solve(microenvironment&, index_t) override {}
	real_t get_substrate_density(index_t, index_t, index_t, index_t) const override { return 0; }
	real_t& get_substrate_density(index_t, index_t, index_t, index_t) override
	{
		static real_t dummy = 0;
		return dummy;
	}
	void reinitialize_dirichlet(microenvironment&) override {}
	void recompute_positional_data(microenvironment&) override {}
};

// test_diffusion_solver.cpp:13-34: timestep 5, D = {4, 2}, decay = {5, 3}, initial 1
std::unique_ptr<microenvironment> default_microenv(const cartesian_mesh& mesh)
{
	auto m = std::make_unique<microenvironment>(mesh, 2, 5.0);
	m->diffusion_coefficients[0] = 4, m->diffusion_coefficients[1] = 2;
	m->decay_rates[0] = 5, m->decay_rates[1] = 3;
	m->initial_conditions[0] = 1, m->initial_conditions[1] = 1;
	return m;
}

// ---- registry (no GPU)

void registry_present_solvers()
{
	auto& registry = solver_registry::instance();
	EXPECT(registry.get("gb300_solver") != nullptr);
	EXPECT(registry.get("gb300_solver_fp32") != nullptr);
}

void registry_get_and_set()
{
	solver_registry registry;
	EXPECT(registry.register_factory("solver_x", []() { return std::make_unique<mock_solver>(); }));
	EXPECT(registry.get("solver_x") != nullptr);
	EXPECT(!registry.register_factory("solver_x", []() { return std::make_unique<mock_solver>(); }));
	EXPECT(registry.get("solver_y") == nullptr);
}

void mesh_geometry()
{
	const cartesian_mesh mesh(3, { 0, 0, 0 }, { 210, 200, 190 }, { 20, 20, 20 });
	EXPECT(mesh.grid_shape[0] == 11 && mesh.grid_shape[1] == 10 && mesh.grid_shape[2] == 10);
	EXPECT(mesh.voxel_volume() == 8000);
	const real_t p[3] = { 39.999, 0.0, 199.0 };
	auto v = mesh.voxel_position(p);
	EXPECT(v[0] == 1 && v[1] == 0 && v[2] == 9);
}

// ---- GPU

// DiffusionSolverTest.Uniform{1,2,3}D through the plugin: one solve step of a
// uniform field with no Dirichlet, bulk or agents is one diffusion step.
void uniform(int dims, std::array<sindex_t, 3> maxs, real_t e0, real_t e1, const char* registry_name)
{
	const cartesian_mesh mesh(dims, { 0, 0, 0 }, maxs, { 20, 20, 20 });
	auto m = default_microenv(mesh);
	m->solver = solver_registry::instance().get(registry_name);
	m->solver->initialize(*m);
	m->run_single_timestep();
	m->solver->transfer_to_host(*m);
	const real_t tol = std::strcmp(registry_name, "gb300_solver") == 0 ? 1e-6 : 1e-6 + 1e-5 * std::fabs(e0);
	for (index_t z = 0; z < mesh.grid_shape[2]; z++)
		for (index_t y = 0; y < mesh.grid_shape[1]; y++)
			for (index_t x = 0; x < mesh.grid_shape[0]; x++)
			{
				EXPECT_NEAR(m->solver->get_substrate_density(0, x, y, z), e0, tol);
				EXPECT_NEAR(m->solver->get_substrate_density(1, x, y, z), e1, tol);
			}
}

void uniform_all()
{
	for (const char* name : { "gb300_solver", "gb300_solver_fp32" })
	{
		uniform(1, { 80, 0, 0 }, 0.03846154, 0.0625, name);
		uniform(2, { 800, 800, 0 }, 0.0054869675, 0.013840831, name);
		uniform(3, { 200, 200, 200 }, 0.0012299563, 0.0046296306, name);
	}
}

// A boundary condition set before initialize holds on its face after a step;
// a changed value reaches the device through reinitialize_dirichlet
// (microenvironment::update_dirichlet_conditions, microenvironment.cpp:255).
void dirichlet_boundary_and_reinitialize()
{
	const cartesian_mesh mesh(2, { 0, 0, 0 }, { 100, 60, 0 }, { 20, 20, 20 });
	auto m = default_microenv(mesh);
	m->dirichlet_min_boundary_values[0] = std::make_unique<real_t[]>(2);
	m->dirichlet_min_boundary_conditions[0] = std::make_unique<bool[]>(2);
	m->dirichlet_min_boundary_values[0][0] = 7.5;
	m->dirichlet_min_boundary_conditions[0][0] = true;
	m->dirichlet_min_boundary_conditions[0][1] = false;
	m->solver = std::make_unique<kernels::gb300_solver::gb300_solver>();
	m->solver->initialize(*m);
	m->run_single_timestep();
	m->solver->transfer_to_host(*m);
	for (index_t y = 0; y < 3; y++)
	{
		EXPECT(m->solver->get_substrate_density(0, 0, y, 0) == 7.5);
		EXPECT(m->solver->get_substrate_density(1, 0, y, 0) != 7.5);
	}
	m->dirichlet_min_boundary_values[0][0] = 2.25;
	m->solver->reinitialize_dirichlet(*m);
	m->run_single_timestep();
	m->solver->transfer_to_host(*m);
	for (index_t y = 0; y < 3; y++)
		EXPECT(m->solver->get_substrate_density(0, 0, y, 0) == 2.25);
}

// Densities written through the mutable accessor reach the device with
// transfer_to_device.  D = 0 and no decay make a diffusion step the identity.
void transfer_round_trip()
{
	const cartesian_mesh mesh(1, { 0, 0, 0 }, { 60, 0, 0 }, { 20, 20, 20 });
	auto m = std::make_unique<microenvironment>(mesh, 1, 0.01);
	m->diffusion_coefficients[0] = 0, m->decay_rates[0] = 0, m->initial_conditions[0] = 0;
	m->solver = std::make_unique<kernels::gb300_solver::gb300_solver>();
	m->solver->initialize(*m);
	m->solver->get_substrate_density(0, 1, 0, 0) = 3.0;
	m->solver->transfer_to_device(*m);
	m->run_single_timestep();
	m->solver->transfer_to_host(*m);
	EXPECT(m->solver->get_substrate_density(0, 0, 0, 0) == 0.0);
	EXPECT(m->solver->get_substrate_density(0, 1, 0, 0) == 3.0);
	EXPECT(m->solver->get_substrate_density(0, 2, 0, 0) == 0.0);
}

// Agents with the reference's implicit update (cell_solver.cpp:51-244), on an
// identity diffusion (D = 0, no decay): two agents share voxel 1 (a ballot
// conflict), one sits in voxel 2; then the agent in voxel 2 moves to voxel 0 and
// recompute_positional_data rebuilds the ballot.
void agents_secretion_and_move()
{
	const cartesian_mesh mesh(1, { 0, 0, 0 }, { 60, 0, 0 }, { 20, 20, 20 });
	auto m = std::make_unique<microenvironment>(mesh, 1, 0.01);
	m->diffusion_coefficients[0] = 0, m->decay_rates[0] = 0, m->initial_conditions[0] = 1.0;
	m->compute_internalized_substrates = true;
	m->agents = std::make_unique<agent_data>(1, 1);
	const real_t xs[3] = { 25.0, 35.0, 45.0 };
	const real_t sec[3] = { 2.0, 0.5, 1.0 }, upt[3] = { 0.25, 3.0, 0.75 };
	for (int i = 0; i < 3; i++)
	{
		const index_t k = m->agents->add();
		m->agents->positions[k] = xs[i];
		m->agents->secretion_rates[k] = sec[i];
		m->agents->saturation_densities[k] = 4.0;
		m->agents->uptake_rates[k] = upt[i];
		m->agents->net_export_rates[k] = 0.1 * (i + 1);
		m->agents->volumes[k] = 1000.0 + 500.0 * i;
	}
	m->solver = std::make_unique<kernels::gb300_solver::gb300_solver>();
	m->solver->initialize(*m);
	m->run_single_timestep();
	m->solver->transfer_to_host(*m);

	const real_t dt = 0.01, Vv = 8000.0;
	auto num = [&](int i) { return sec[i] * 4.0 * dt * m->agents->volumes[i] / Vv; };
	auto den = [&](int i) { return (sec[i] + upt[i]) * dt * m->agents->volumes[i] / Vv; };
	auto fac = [&](int i) { return m->agents->net_export_rates[i] * dt / Vv; };
	// voxel 1 holds agents 0 and 1, voxel 2 agent 2
	const real_t d1 = (1.0 + (num(0) + num(1))) / (1.0 + den(0) + den(1)) + (fac(0) + fac(1));
	const real_t d2 = (1.0 + num(2)) / (1.0 + den(2)) + fac(2);
	EXPECT_NEAR(m->solver->get_substrate_density(0, 0, 0, 0), 1.0, 0.0);
	EXPECT_NEAR(m->solver->get_substrate_density(0, 1, 0, 0), d1, 1e-15);
	EXPECT_NEAR(m->solver->get_substrate_density(0, 2, 0, 0), d2, 1e-15);
	// a conflict anywhere takes the two-pass internalized update for every agent
	const real_t i0 = -Vv * (num(0) - d1 * den(0) + fac(0));
	const real_t i2 = -Vv * (num(2) - d2 * den(2) + fac(2));
	EXPECT_NEAR(m->agents->internalized_substrates[0], i0, 1e-12 * std::fabs(i0));
	EXPECT_NEAR(m->agents->internalized_substrates[2], i2, 1e-12 * std::fabs(i2));

	// agent 2 moves to voxel 0
	m->agents->positions[2] = 5.0;
	m->solver->recompute_positional_data(*m);
	m->run_single_timestep();
	m->solver->transfer_to_host(*m);
	const real_t d0 = (1.0 + num(2)) / (1.0 + den(2)) + fac(2);
	EXPECT_NEAR(m->solver->get_substrate_density(0, 0, 0, 0), d0, 1e-15);
	EXPECT_NEAR(m->solver->get_substrate_density(0, 2, 0, 0), d2, 0.0); // untouched since
}

struct test_case
{
	const char* name;
	std::function<void()> fn;
	bool gpu;
};

} // namespace

int main(int argc, char** argv)
{
	const bool cpu_only = argc > 1 && std::strcmp(argv[1], "--cpu") == 0;
	const test_case tests[] = {
		{ "SolverRegistryTest.CheckPresentSolvers", registry_present_solvers, false },
		{ "SolverRegistryTest.GetAndSet", registry_get_and_set, false },
		{ "MeshTest.Geometry", mesh_geometry, false },
		{ "Gb300SolverTest.Uniform", uniform_all, true },
		{ "Gb300SolverTest.DirichletBoundaryAndReinitialize", dirichlet_boundary_and_reinitialize, true },
		{ "Gb300SolverTest.TransferRoundTrip", transfer_round_trip, true },
		{ "Gb300SolverTest.AgentsSecretionAndMove", agents_secretion_and_move, true },
	};
	int ran = 0;
	for (const auto& t : tests)
	{
		if (t.gpu && cpu_only)
			continue;
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
