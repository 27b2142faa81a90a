// pcg_internal.cuh -- shared definitions of the GB300 BioFVM backend.
//
// Device data layout (chosen for the sweeps, not copied from the reference):
//   field[s][z][y][x], each x-row padded to `pitch` elements so that every row
//   starts on a 32-byte sector boundary.  Element (s,x,y,z) lives at
//   ((s*nz + z)*ny + y)*pitch + x.  The reference keeps substrates interleaved
//   (s fastest, diffusion_solver.h:64-83); host transfers convert between the two.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/physicore_gb300.h"

namespace pcg {

// ------------------------------------------------------------------ errors

void set_error(const std::string& msg);
int fail(int code, const std::string& msg);

#define PCG_CUDA_TRY(expr)                                                                                   \
	do                                                                                                       \
	{                                                                                                        \
		cudaError_t err__ = (expr);                                                                          \
		if (err__ != cudaSuccess)                                                                            \
			return ::pcg::fail(PCG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(err__));         \
	} while (0)

// Device error word bits, set by kernels with atomicOr instead of trapping.
enum : uint32_t
{
	DEV_ERR_AGENT_OUTSIDE = 1u << 0, // an active agent's voxel index fell outside the grid
	DEV_ERR_WAIT_TIMEOUT = 1u << 1,  // a bounded mbarrier wait ran out
	DEV_ERR_DIRICHLET_INDEX = 1u << 2,
	DEV_ERR_BAD_TILE = 1u << 3,
};

// ------------------------------------------------------------------ kernel ids

enum KernelId : int
{
	K_SWEEP_X = 0,
	K_SWEEP_Y,
	K_SWEEP_Z,
	K_DIRICHLET_FACES,
	K_DIRICHLET_INTERIOR,
	K_BULK,
	K_CELLS_LOCATE,
	K_CELLS_BALLOT,
	K_CELLS_REDUCE,
	K_CELLS_APPLY,
	K_CELLS_INTERNALIZE,
	K_CELLS_RELEASE,
	K_MASS,
	K_LAYOUT,
	K_COUNT
};

const char* kernel_name(int id);

// ------------------------------------------------------------------ launch geometry

constexpr int kSweepLanes = 32;        // lines per y/z tile (one warp)
constexpr int kSweepXRows = 32;        // rows per x tile (one warp)
constexpr uint64_t kMaxSmemBytes = 227 * 1024;

// ------------------------------------------------------------------ argument blocks

// One Thomas sweep along y or z over a set of tiles.  A tile is `lanes`
// consecutive x positions of every line of one (s, outer) pair.
struct SweepYZArgs
{
	void* field;
	const void* coef;     // per substrate: B[n], E[n] (E[0] = 0, E[i] = e_{i-1}), padded to coef_pitch
	const void* coef_c;   // c[s]
	uint64_t coef_pitch;  // elements between the B tables of consecutive substrates (E follows B)
	uint64_t n;           // line length
	uint64_t nx;
	uint64_t line_stride; // elements between consecutive points of a line
	uint64_t outer_count; // z (y sweep) or y (z sweep)
	uint64_t outer_stride;
	uint64_t plane;       // elements per substrate
	uint64_t xblocks;
	uint64_t tiles;
	uint32_t* err;
};

// One Thomas sweep along x.  A tile is up to `rows` consecutive rows of one substrate.
struct SweepXArgs
{
	void* field;
	const void* coef;
	const void* coef_c;
	uint64_t coef_pitch;
	uint64_t n;           // nx
	uint64_t pitch;       // row pitch of the field (elements)
	uint64_t rows;        // rows per substrate (ny*nz)
	uint64_t rblocks;     // tiles per substrate
	uint64_t tiles;
	uint64_t smem_pitch;  // shared-memory row pitch (elements)
	uint32_t* err;
};

// ------------------------------------------------------------------ context

struct DeviceBuffer
{
	void* ptr = nullptr;
	size_t bytes = 0;
};

struct Context;

int dalloc(Context* c, DeviceBuffer& b, size_t bytes);
void dfree(DeviceBuffer& b);

struct KernelStat
{
	uint64_t launches = 0;
	double total_ms = 0;
	double bytes = 0;
};

struct Context
{
	int device = 0;
	int precision = PCG_FP32;
	size_t wsize = 4; // bytes per field element
	cudaStream_t own_stream = nullptr;
	cudaStream_t stream = nullptr;

	// mesh
	int dims = 0;
	int64_t bbmin[3] = { 0, 0, 0 }, bbmax[3] = { 0, 0, 0 };
	uint64_t voxel[3] = { 0, 0, 0 };
	uint64_t n[3] = { 1, 1, 1 };
	bool mesh_set = false;

	// substrates
	uint64_t S = 0;
	double dt = 0;
	std::vector<double> D, decay, init;

	// derived layout
	uint64_t pitch = 0; // row pitch (elements)
	uint64_t plane = 0; // elements per substrate = nz*ny*pitch
	uint64_t V = 0;

	// device state
	bool initialized = false;
	bool recompute_cells = true;
	DeviceBuffer field;
	DeviceBuffer coef[3];
	DeviceBuffer coef_c[3];
	uint64_t coef_pitch[3] = { 0, 0, 0 };
	DeviceBuffer err;      // uint32 device error word
	DeviceBuffer flags;    // uint32 [4]: [0] ballot conflict
	DeviceBuffer mass;     // double [S]
	DeviceBuffer staging;  // layout conversion

	// Dirichlet
	uint64_t K = 0;
	std::vector<uint64_t> h_dir_voxels;
	std::vector<double> h_dir_values;
	std::vector<uint8_t> h_dir_conds;
	DeviceBuffer dir_offsets; // uint64 [K] element offset inside a substrate plane
	DeviceBuffer dir_values;  // real [K*S]
	DeviceBuffer dir_conds;   // uint8 [K*S]
	bool face_on[3][2] = { { false, false }, { false, false }, { false, false } };
	std::vector<double> h_face_values[3][2];
	std::vector<uint8_t> h_face_conds[3][2];
	DeviceBuffer face_values; // real [6*S]
	DeviceBuffer face_conds;  // uint8 [6*S]
	bool dirichlet_dirty = true;

	// bulk
	int bulk_mode = PCG_BULK_NONE;
	std::vector<double> h_bulk[3];
	DeviceBuffer bulk[3]; // real tables: supply, uptake, target (S or S*plane)
	bool bulk_dirty = true;

	// agents
	uint64_t A = 0;
	bool compute_internalized = false;
	DeviceBuffer a_pos, a_sec, a_sat, a_upt, a_net, a_vol, a_active, a_internal, a_frac;
	// cell scratch
	DeviceBuffer a_foff;                  // uint32 [A]: offset of the agent's voxel inside a plane
	DeviceBuffer a_num, a_den, a_fac;     // real [A*S]
	DeviceBuffer a_rnum, a_rden, a_rfac;  // real [A*S]
	DeviceBuffer owner;                   // uint32 [plane]: winning agent per voxel
	DeviceBuffer counts;                  // uint32 [plane]: active agents per voxel

	// measurement
	bool timing = false;
	KernelStat stats[K_COUNT];
	uint64_t launches = 0;
	std::vector<cudaEvent_t> event_pool;
	struct PendingTiming
	{
		int kid;
		cudaEvent_t a, b;
	};
	std::vector<PendingTiming> pending;
};

// Launch bookkeeping: every kernel launch goes through begin/end so that the
// context can count launches and (optionally) time them with CUDA events.
void launch_begin(Context* c, int kid, double bytes, cudaEvent_t* ev);
void launch_end(Context* c, int kid, cudaEvent_t ev);
void collect_timings(Context* c);

// ------------------------------------------------------------------ kernel launchers (defined in .cu files)

int launch_sweep_x(Context* c);
int launch_sweep_yz(Context* c, int axis);
int launch_dirichlet(Context* c);
int launch_bulk(Context* c);
int launch_cells(Context* c, bool recompute);
int launch_release(Context* c, uint64_t agent);
int launch_mass(Context* c, double* dev_out);
int launch_to_host_layout(Context* c, void* dst, int layout, int dtype);
int launch_from_host_layout(Context* c, const void* src, int layout, int dtype);
int launch_fill_initial(Context* c);

uint64_t sweep_yz_smem_bytes(const Context* c, int axis);
uint64_t sweep_x_smem_bytes(const Context* c);
uint64_t sweep_x_smem_pitch(const Context* c);

} // namespace pcg

// ------------------------------------------------------------------ device helpers

#ifdef __CUDACC__
namespace pcg::dev {

// Bounded mbarrier wait: gives up after kWaitNs nanoseconds of %globaltimer time
// (a tile load takes microseconds), and the caller flags DEV_ERR_WAIT_TIMEOUT.
constexpr uint64_t kWaitNs = 50ull * 1000 * 1000;

__device__ __forceinline__ uint64_t global_ns()
{
	uint64_t t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
	return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
				 : "memory");
}

// Returns true when the phase with parity `phase` completed within the limit.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase)
{
	const uint32_t addr = smem_addr(bar);
	const uint64_t t0 = global_ns();
	for (;;)
	{
		uint32_t done;
		asm volatile(
			"{\n\t.reg .pred p;\n\t"
			"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(done)
			: "r"(addr), "r"(phase)
			: "memory");
		if (done)
			return true;
		if (global_ns() - t0 > kWaitNs)
			return false;
	}
}

// Bulk copy global -> shared, completing on `bar` (size and both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
	asm volatile(
		"cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
			smem_addr(dst)),
		"l"(src), "r"(bytes), "r"(smem_addr(bar))
		: "memory");
}

// Bulk copy shared -> global in the calling thread's bulk async-group.
__device__ __forceinline__ void bulk_s2g(void* dst, const void* src, uint32_t bytes)
{
	asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
				 "r"(bytes)
				 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Makes generic-proxy shared-memory writes visible to the async (bulk copy) proxy.
__device__ __forceinline__ void fence_proxy_async_smem()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

} // namespace pcg::dev
#endif
