// diffuse.cpp -- reads a PhysiCell_settings.xml file, builds the microenvironment
// through the builder and the solver registry, places agents and steps the
// simulation to <max_time>, writing VTK image files at a fixed interval: the
// caller path of the reference's example (reactions-diffusion/biofvm/examples/
// diffuse.cpp:15-155) on the gb300 solver.
//
//   diffuse [settings.xml] [--output DIR] [--agents FILE] [--steps N]
//           [--interval T] [--transfer-every-step] [--solver NAME]
//
// --agents reads agents from a text file instead of the built-in groups:
//   A S
//   then per agent: x y z volume, S secretion rates, S saturation densities,
//   S uptake rates, S net export rates (whitespace separated, any strtod form).
// --steps N runs N steps instead of max_time / dt.  --interval sets the output
// interval (default 0.1 time units; outputs also go out at t = 0 and after the
// last step).  --transfer-every-step moves the field to and from the device
// around every step, as the reference's example loop does; by default the
// field stays on the device and is read only for outputs.  --solver overrides
// the settings file's <solver><name>.
//
// Prints one line per output and a final summary line with the step count, the
// time spent stepping and writing, and voxel-substrate-steps per second.
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <memory>
#include <random>
#include <string>
#include <vector>

#include "../csrc/host/config_reader.h"
#include "../csrc/host/microenvironment.h"
#include "../csrc/host/microenvironment_builder.h"

using namespace physicore;
using namespace physicore::biofvm;

namespace {

struct options
{
	std::string settings = "settings.xml";
	std::string output = "output";
	std::string agents;
	std::string solver;
	long long steps = -1;
	double interval = 0.1;
	bool transfer_every_step = false;
};

options parse_args(int argc, char** argv)
{
	options o;
	for (int i = 1; i < argc; i++)
	{
		const std::string a = argv[i];
		auto value = [&]() -> std::string {
			if (i + 1 >= argc)
				throw std::runtime_error("missing value after " + a);
			return argv[++i];
		};
		if (a == "--output")
			o.output = value();
		else if (a == "--agents")
			o.agents = value();
		else if (a == "--steps")
			o.steps = std::stoll(value());
		else if (a == "--interval")
			o.interval = std::stod(value());
		else if (a == "--solver")
			o.solver = value();
		else if (a == "--transfer-every-step")
			o.transfer_every_step = true;
		else if (!a.empty() && a[0] == '-')
			throw std::runtime_error("unknown option " + a);
		else
			o.settings = a;
	}
	return o;
}

// Builds like microenvironment::create_from_config, with the output directory
// and solver name of the command line.
std::unique_ptr<microenvironment> load(const options& o)
{
	const physicell_config c = parse_physicell_config(o.settings);
	microenvironment_builder b;
	configure_from(b, c);
	b.set_output_dir(o.output);
	b.select_solver(!o.solver.empty() ? o.solver : !c.solver.name.empty() ? c.solver.name : "gb300_solver");
	return b.build();
}

// Agents in three spherical clusters with their own rates for the first two
// densities (zero for the others).
void place_default_agents(microenvironment& m)
{
	struct cluster
	{
		std::array<real_t, 3> center;
		real_t radius, volume;
		std::array<real_t, 2> secretion, saturation, uptake;
		int count;
	};
	const cluster clusters[] = {
		{ { -450.0, -150.0, 0.0 }, 160.0, 2300.0, { 5.0, 2.0 }, { 40.0, 7.0 }, { 300.0, 150.0 }, 40 },
		{ { 100.0, 250.0, 0.0 }, 200.0, 2600.0, { 80.0, 60.0 }, { 30.0, 4.5 }, { 0.1, 0.05 }, 36 },
		{ { 500.0, -300.0, 0.0 }, 110.0, 1900.0, { 350.0, 420.0 }, { 20.0, 3.0 }, { 0.2, 0.12 }, 28 },
	};
	std::mt19937_64 rng(2024);
	std::uniform_real_distribution<real_t> unit(-1.0, 1.0);
	agent_data& a = *m.agents;
	const index_t S = m.substrates_count, dims = m.mesh.dims;
	for (const cluster& c : clusters)
		for (int k = 0; k < c.count; k++)
		{
			const index_t i = a.add();
			for (index_t d = 0; d < dims; d++)
			{
				// inside the domain: clamp to [min, max) of the mesh
				const real_t lo = (real_t)m.mesh.bounding_box_mins[d], hi = (real_t)m.mesh.bounding_box_maxs[d];
				real_t p = c.center[d] + unit(rng) * c.radius;
				p = std::min(std::max(p, lo), std::nextafter(hi, lo));
				a.positions[i * dims + d] = p;
			}
			for (index_t s = 0; s < S && s < 2; s++)
			{
				a.secretion_rates[i * S + s] = c.secretion[s];
				a.saturation_densities[i * S + s] = c.saturation[s];
				a.uptake_rates[i * S + s] = c.uptake[s];
			}
			a.volumes[i] = c.volume;
		}
}

void read_agents(microenvironment& m, const std::string& path)
{
	std::ifstream f(path);
	if (!f)
		throw std::runtime_error("cannot open agents file " + path);
	auto next = [&]() -> double {
		std::string tok;
		if (!(f >> tok))
			throw std::runtime_error("agents file " + path + " ends early");
		return std::strtod(tok.c_str(), nullptr);
	};
	const auto A = (index_t)next(), S = (index_t)next();
	if (S != m.substrates_count)
		throw std::runtime_error("agents file substrate count does not match the settings");
	agent_data& a = *m.agents;
	const index_t dims = m.mesh.dims;
	for (index_t k = 0; k < A; k++)
	{
		const index_t i = a.add();
		for (index_t d = 0; d < 3; d++)
		{
			const double p = next();
			if (d < dims)
				a.positions[i * dims + d] = p;
		}
		a.volumes[i] = next();
		for (auto* v : { &a.secretion_rates, &a.saturation_densities, &a.uptake_rates, &a.net_export_rates })
			for (index_t s = 0; s < S; s++)
				(*v)[i * S + s] = next();
	}
}

} // namespace

int main(int argc, char** argv)
{
	try
	{
		const options o = parse_args(argc, argv);
		std::cout << "[diffuse] Loading configuration from: " << o.settings << std::endl;
		std::unique_ptr<microenvironment> m = load(o);
		m->print_info(std::cout);
		if (!o.agents.empty())
			read_agents(*m, o.agents);
		else
			place_default_agents(*m);

		const real_t dt = m->diffusion_timestep;
		const long long steps = o.steps >= 0 ? o.steps : (long long)std::llround(m->simulation_time / dt);
		const double vss_per_step = (double)m->mesh.voxel_count() * (double)m->substrates_count;

		m->solver->initialize(*m);
		m->serialize_state(0.0);
		std::cout << "[diffuse] Running " << steps << " steps of " << dt << " " << m->time_units << " ("
				  << m->agents->agents_count << " agents)" << std::endl;

		using clock = std::chrono::steady_clock;
		std::chrono::duration<double> step_time { 0 }, write_time { 0 }, step_total { 0 }, write_total { 0 };
		real_t next_output = o.interval;
		for (long long k = 1; k <= steps; k++)
		{
			const real_t t = dt * (real_t)k;
			const bool output = t + 1e-12 >= next_output || k == steps;
			const auto t0 = clock::now();
			if (o.transfer_every_step)
				m->solver->transfer_to_device(*m);
			m->run_single_timestep();
			if (o.transfer_every_step || output)
				m->solver->transfer_to_host(*m); // synchronises: the step is done
			step_time += clock::now() - t0;
			if (output)
			{
				while (next_output <= t + 1e-12)
					next_output += o.interval;
				const auto w0 = clock::now();
				m->serialize_state(t);
				write_time = clock::now() - w0;
				write_total += write_time;
				step_total += step_time;
				std::cout << "[diffuse] t=" << t << " diffusion runtime: " << step_time.count()
						  << " s serialization runtime: " << write_time.count() << " s" << std::endl;
				step_time = std::chrono::duration<double> { 0 };
			}
		}
		std::printf("[diffuse] done: steps=%lld step_s=%.6f write_s=%.6f vss_per_s=%.6e\n", steps, step_total.count(),
					write_total.count(), step_total.count() > 0 ? vss_per_step * (double)steps / step_total.count() : 0.0);
		return 0;
	}
	catch (const std::exception& e)
	{
		std::cerr << "[diffuse] Error: " << e.what() << std::endl;
		return 1;
	}
}
