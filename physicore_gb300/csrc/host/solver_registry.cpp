// solver_registry.cpp -- see solver_registry.h.  The GB300 solvers attach
// themselves when the library loads, as the reference's backends do through its
// static attachment point (src/solver_registry.cpp:38-52).
#include "solver_registry.h"

#include "gb300_solver.h"

namespace physicore::biofvm {

bool solver_registry::register_factory(std::string solver_name, solver_factory_func_t&& f)
{
	auto [it, emplaced] = factory_registry.try_emplace(std::move(solver_name), std::move(f));
	return emplaced;
}

solver_ptr solver_registry::get(const std::string& solver_name)
{
	auto it = factory_registry.find(solver_name);
	if (it == factory_registry.end())
		return nullptr;
	return it->second();
}

solver_registry& solver_registry::instance()
{
	static solver_registry r;
	return r;
}

namespace {
struct attachment_point
{
	attachment_point() { kernels::gb300_solver::gb300_solver::attach_to_registry(); }
};
const attachment_point ap;
} // namespace

} // namespace physicore::biofvm
