// gb300_solver.h -- a solver plugin backed by the GB300 C ABI
// (include/physicore_gb300.h), the class a PhysiCore build registers next to its
// OpenMP and Thrust backends (reactions-diffusion/biofvm/kernels/*/register_solver.*).
//
// Semantics follow the reference's device backend (thrust_solver.cpp:7-66): the
// field lives on the GPU; get_substrate_density reads a host mirror that is valid
// after transfer_to_host; transfer_to_device uploads that mirror and the agents'
// positions and activity.  The context is created on the first initialize (so that
// the registry can construct the solver without touching a GPU).  A bulk functor
// is tabulated per voxel at initialize and on refresh_bulk.
#pragma once

#include <vector>

#include "../../../include/physicore_gb300.h"
#include "microenvironment.h"
#include "solver.h"

namespace physicore::biofvm::kernels::gb300_solver {

class gb300_solver : public solver
{
public:
	explicit gb300_solver(int precision = PCG_FP64, int device = 0) : precision_(precision), device_(device) {}
	~gb300_solver() override;

	void initialize(microenvironment& m) override;
	void solve(microenvironment& m, index_t iterations) override;
	real_t get_substrate_density(index_t s, index_t x, index_t y, index_t z) const override;
	real_t& get_substrate_density(index_t s, index_t x, index_t y, index_t z) override;
	void transfer_to_device(microenvironment& m) override;
	void transfer_to_host(microenvironment& m) override;
	void reinitialize_dirichlet(microenvironment& m) override;
	void recompute_positional_data(microenvironment& m) override;

	// Re-tabulates the microenvironment's bulk functor on the device.
	void refresh_bulk(microenvironment& m);

	// The underlying context (for batching several solvers with pcg_batch_create).
	pcg_context* context() const { return ctx_; }

	// The device field in planar order [s][z][y][x], FP64, one bulk copy (the
	// image serializer's read; the host mirror is not involved).
	void read_field_planar(real_t* out) const;

	// Registers "gb300_solver" (FP64) and "gb300_solver_fp32".
	static void attach_to_registry();

private:
	void upload_dirichlet(microenvironment& m);
	void upload_agents(microenvironment& m);
	void refresh_agents(microenvironment& m); // positions/activity, or everything if agents were added
	std::size_t index(index_t s, index_t x, index_t y, index_t z) const;

	int precision_, device_;
	pcg_context* ctx_ = nullptr;
	bool initialized_ = false;
	index_t S_ = 0, n_[3] = { 1, 1, 1 };
	index_t agents_uploaded_ = 0; // agent count the context holds
	std::vector<real_t> host_; // interleaved mirror: s + S * (x + nx * (y + ny * z))
};

struct gb300_solver_fp32 : gb300_solver
{
	gb300_solver_fp32() : gb300_solver(PCG_FP32) {}
};

} // namespace physicore::biofvm::kernels::gb300_solver
