// solver.h -- the solver plugin interface, with the reference's methods and meaning
// (reactions-diffusion/biofvm/include/biofvm/solver.h:12-39).
#pragma once

#include <memory>

#include "types.h"

namespace physicore::biofvm {

struct microenvironment;

class solver
{
public:
	// Sets initial values (such as substrate densities) in the microenvironment
	virtual void initialize(microenvironment& m) = 0;

	// Solves the diffusion-decay equations (and Dirichlet, bulk, cells) for a number of iterations
	virtual void solve(microenvironment& m, index_t iterations) = 0;

	// The substrate density at a voxel
	virtual real_t get_substrate_density(index_t s, index_t x, index_t y, index_t z) const = 0;
	virtual real_t& get_substrate_density(index_t s, index_t x, index_t y, index_t z) = 0;

	// Moves data to/from the device (no-ops for host solvers)
	virtual void transfer_to_device([[maybe_unused]] microenvironment& m) {}
	virtual void transfer_to_host([[maybe_unused]] microenvironment& m) {}

	// Re-reads the Dirichlet conditions after they were modified
	virtual void reinitialize_dirichlet(microenvironment& m) = 0;

	// Re-reads agent positions after another module moved them
	virtual void recompute_positional_data(microenvironment& m) = 0;

	virtual ~solver() = default;
};

using solver_ptr = std::unique_ptr<solver>;

} // namespace physicore::biofvm
