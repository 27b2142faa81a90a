// pcg_internal.cuh -- shared definitions of the GB300 BioFVM backend.
//
// Device field layout: the reference's interleaved order (s fastest, then x, y, z;
// openmp_solver/src/diffusion_solver.h:64-83) with every x-row padded to `pitch`
// elements, pitch*sizeof(T) a multiple of 32 bytes so rows start on DRAM sectors.
// Element (s,x,y,z) lives at (z*ny + y)*pitch + x*S + s.  Keeping a voxel's
// substrates adjacent makes every agent touch one sector per voxel (S*4 <= 32 B for
// S <= 8 in FP32); the y/z sweeps tile the merged (x,s) run of a row, and the x
// sweep walks whole rows with S independent recurrences per thread.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <memory>
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
	K_CELLS_CLEAR,
	K_MASS_CHECK,
	K_CELLS_GROUP,
	K_SWEEP_XY,
	K_COUNT
};

const char* kernel_name(int id);

// ------------------------------------------------------------------ launch geometry

constexpr int kLanes = 32;           // lines per y/z tile, rows per x tile (one warp per CTA)
constexpr int kStages = 2;           // shared-memory ring depth of the persistent sweeps
constexpr uint64_t kMaxSmemBytes = 227 * 1024;
constexpr uint64_t kCoefSmemLimit = 64 * 1024; // larger coefficient tables stay in global memory
constexpr uint64_t kBlockPoints = 8;           // line points per pipelined solver block
constexpr uint64_t kXTileBytes = 32 * 1024;    // shared memory of a substrate-mapped x tile

__host__ __device__ constexpr uint64_t round_up(uint64_t v, uint64_t m) { return (v + m - 1) / m * m; }

// Values per agent row of the cell terms (num, den and fac of S substrates side by
// side, cells_device.cuh): 3 S values of w bytes in whole 16-byte units, so that a
// gather of one agent's terms touches one short run of memory, not three rows.
__host__ __device__ constexpr uint64_t term_stride(uint64_t S, uint64_t w) { return round_up(3 * S * w, 16) / w; }
__host__ __device__ constexpr int gcd_i(int a, int b) { return b == 0 ? a : gcd_i(b, a % b); }
// Elements per x-sweep vector group: the smallest multiple of both S and a 16-byte chunk.
__host__ __device__ constexpr int group_elems(int S, int vn) { return S <= 8 ? S / gcd_i(S, vn) * vn : vn; }

// ------------------------------------------------------------------ argument block

// A Thomas sweep over one axis.  The coefficient table of the axis is
// [B | E | C]: B[i*S+s] = b'_i, E[i*S+s] = e_{i-1} (E = 0 for i = 0), each
// padded to coef_len elements, then C[s] = c padded to a 16-byte multiple.
struct SweepArgs
{
	void* field;
	const void* coef;
	uint64_t coef_len;    // elements of one padded B or E table
	uint64_t coef_elems;  // elements of the whole [B | E | C] table
	uint32_t S;
	uint32_t n;           // line length
	uint64_t row_len;     // nx*S: elements of one row
	uint64_t pitch;       // row pitch of the field (elements)
	uint64_t tiles;
	// y/z sweeps: a tile is 32 consecutive (x,s) elements of all n points of a line set
	uint64_t line_stride; // elements between consecutive points of a line
	uint64_t outer_stride;
	uint64_t xblocks;
	uint32_t box_rows;    // line points per TMA box (<= 256)
	uint32_t boxes;       // boxes per tile (boxes * box_rows >= n)
	uint64_t comp_off;    // compressed coefficient tables (elements into coef)
	uint64_t blo_off;     // FP32: full table of the multipliers' lo parts (elements into coef)
	uint32_t head;        // head points of the compressed tables
	// x sweep: a tile is rows_per_tile whole rows
	uint64_t rows;        // ny*nz
	uint64_t smem_pitch;  // shared-memory row pitch (elements); in 16-byte chunks == threads per row (mod 8)
	uint32_t rows_per_tile;
	uint32_t* err;
	uint32_t* ticket; // tile counter of the launch (zeroed before it), tiles handed out in order
	// y/z, last sweep of a step that also applies Dirichlet: the boundary faces
	// are written into each solved tile before it is stored (FaceArgs in
	// field_device.cuh); face_mask 0 when not fused
	const void* face_values;
	const uint8_t* face_conds;
	uint32_t face_mask;
	uint64_t nx, ny, nz;
	// mass check (kernels instantiated with it): FP64 totals [before S | after S];
	// the x sweep adds its inputs, the last sweep its outputs (x as well when the
	// mesh is 1-D)
	double* mc_tot;
	uint32_t mc_x_out;
};

// ------------------------------------------------------------------ context

// Device memory from the stream-ordered allocator: allocated and freed on `stream`
// (a stream that outlives the buffer), so that freeing never waits for the device.
struct DeviceBuffer
{
	void* ptr = nullptr;
	size_t bytes = 0;
	cudaStream_t stream = nullptr;
	bool carved = false; // a piece of its context's slab: released with the slab
};

struct Context;

int dalloc(Context* c, DeviceBuffer& b, size_t bytes);
// Stream-ordered allocation from the library's pool on `device` (capi.cu), and the
// bytes that pool holds free for reuse.
cudaError_t pool_alloc(void** ptr, size_t bytes, cudaStream_t stream, int device);
uint64_t pool_idle_bytes(int device);
// Four pinned host words (capi.cu) for small device-to-host reads (error words):
// a copy into pinned memory is a plain DMA, whereas a synchronous copy into
// pageable memory goes through driver staging shared by every thread and, queued
// behind other copies, stalls the transfers of all of them.  Null when pinned
// memory cannot be had.
uint32_t* pinned_words_get();
void pinned_words_put(uint32_t* w);
// Host wait for the context's stream, asleep rather than spinning (capi.cu).
cudaError_t stream_wait(Context* c);
// Whether the field readback `ticket` of pcg_get_field_async is in host memory,
// without waiting (capi.cu).
int readback_ready(Context* c, uint64_t ticket, bool* done);
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
	int sm_count = 0;
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
	uint64_t row_len = 0; // nx*S
	uint64_t pitch = 0;   // row pitch (elements)
	uint64_t rows = 0;    // ny*nz
	uint64_t V = 0;

	// device state
	bool initialized = false;
	bool recompute_cells = true;
	bool terms_dirty = true; // agent rates or volumes uploaded since the agent terms were computed
	bool words_cleared = false; // err/flags words zeroed on the device
	// bumped by every call that may reallocate a device buffer or change a
	// parameter; batches compare it with the value they captured
	uint64_t generation = 0;
	DeviceBuffer field;
	DeviceBuffer coef[3];
	// TMA tensor maps of the field for the y and z sweeps: the field as a 3-D tensor
	// (x*S+s, y, z) with 32 x (box_rows) boxes along the swept axis
	CUtensorMap tmap[3];
	uint32_t tmap_box_rows[3] = { 0, 0, 0 };
	uint32_t tmap_boxes[3] = { 0, 0, 0 };
	uint64_t coef_len[3] = { 0, 0, 0 };
	uint64_t coef_elems[3] = { 0, 0, 0 };
	uint64_t coef_comp_off[3] = { 0, 0, 0 }; // compressed tables (head rows, constants)
	uint64_t coef_blo_off[3] = { 0, 0, 0 };  // FP32: the full table of the multipliers' lo parts
	uint32_t coef_head[3] = { 0, 0, 0 };     // head points per substrate of the compressed tables
	// One allocation at initialisation sized by estimate_device_bytes, from which
	// the context's buffers are carved in turn (dozens of pool allocations per
	// context cost milliseconds once many contexts come and go, as under a server)
	DeviceBuffer slab;
	size_t slab_used = 0;
	DeviceBuffer err;      // uint32 device error word
	uint32_t* h_words = nullptr; // pinned host words for reading it
	cudaEvent_t ev_block = nullptr; // blocking-sync event for host waits on the stream
	DeviceBuffer tickets;  // uint32 [4]: tile counters of the persistent sweeps ([3]: fused x/y)
	// fused x/y sweeps: on/off (pcg_set_sweep_fusion), slab size, lag, and the
	// segment table and per-slab counters of the current plan
	bool fuse_xy = false;
	uint64_t xy_slab_bytes = 8ull << 20;
	uint32_t xy_lag = 2;
	uint64_t xy_key = 0;
	uint32_t xy_nseg = 0, xy_total = 0, xy_nslab = 0;
	DeviceBuffer xy_segs, xy_done;
	DeviceBuffer flags;    // uint32 [8]: [0] ballot conflict, [1] agents in shared voxels (batches),
	                       // [2..3] and [4] the grouped ballot's counts (cells_device.cuh)
	DeviceBuffer mass;     // double [S]
	// per-step mass check (pcg_set_mass_check): FP64 totals [2 * S] before the
	// first sweep and after the last one, added by the sweeps themselves, and
	// [4 * S]: mass before, mass after, worst residual, the product of the sweep
	// matrices' column sums
	bool mass_check = false;
	uint64_t mass_checked_steps = 0;
	DeviceBuffer mc_tot;
	DeviceBuffer mc_out;
	DeviceBuffer staging;  // layout conversion
	// asynchronous field readback: two staging buffers used in turn, copied to the
	// host on a stream of their own; readback k uses slot k % 2
	DeviceBuffer rb_staging[2];
	cudaStream_t rb_stream = nullptr;
	cudaEvent_t rb_packed[2] = { nullptr, nullptr }, rb_done[2] = { nullptr, nullptr };
	bool rb_pending[2] = { false, false };
	uint64_t rb_issued = 0;

	// Dirichlet
	uint64_t K = 0;
	std::vector<uint64_t> h_dir_voxels;
	std::vector<double> h_dir_values;
	std::vector<uint8_t> h_dir_conds;
	DeviceBuffer dir_offsets; // uint64 [K] field offset of the node's first substrate
	DeviceBuffer dir_values;  // real [K*S]
	DeviceBuffer dir_conds;   // uint8 [K*S]
	bool face_on[3][2] = { { false, false }, { false, false }, { false, false } };
	std::vector<double> h_face_values[3][2];
	std::vector<uint8_t> h_face_conds[3][2];
	DeviceBuffer face_values; // real [6*S]
	DeviceBuffer face_conds;  // uint8 [6*S]

	// bulk
	int bulk_mode = PCG_BULK_NONE;
	std::vector<double> h_bulk[3];
	DeviceBuffer bulk[3]; // real tables: supply, uptake, target ([S] or field-shaped)

	// agents
	uint64_t A = 0;
	bool compute_internalized = false;
	// Agents set before initialize wait here (host copies) and reach the device in
	// initialize, so that an uninitialised context holds no device memory.
	struct HostAgents
	{
		std::vector<double> pos, sec, sat, upt, net, vol;
		std::vector<double> internal, frac; // empty: all zero (cleared on the device, nothing copied)
		std::vector<uint8_t> active;
	};
	std::unique_ptr<HostAgents> staged_agents;
	DeviceBuffer a_pos, a_sec, a_sat, a_upt, a_net, a_vol, a_active, a_internal, a_frac;
	// cell scratch
	DeviceBuffer a_vox;                   // uint32 [A]: linear voxel index (x + nx*(y + ny*z)), or ~0
	DeviceBuffer a_foff;                  // uint32 [A]: field offset of the voxel's first substrate
	DeviceBuffer a_role;                  // uint8 [A]: ballot role (cells_device.cuh)
	DeviceBuffer a_shared;                // uint32 [A]: agents of voxels that hold several
	DeviceBuffer a_rank;                  // uint32 [A]: rank of the agent in its voxel
	DeviceBuffer a_sorted;                // uint2 [A]: (agent, voxel) of shared voxels grouped by voxel
	DeviceBuffer a_writers;               // uint32 [A]: agents that write a voxel (alone or winner)
	// the ballot behind the cached roles, lists and reduced rows: 0 none, 1 the
	// grouped ballot of a single-domain step, 2 a batch's per-warp ballot (their
	// lists and counts differ, so a step of the other kind rebuilds)
	uint8_t ballot_kind = 0;
	uint64_t term_stride = 0;             // values per agent row of a_terms and a_reduced
	DeviceBuffer a_terms;                 // real [A][term_stride]: num, den, fac of the agent (S each)
	DeviceBuffer a_reduced;               // real [A][term_stride]: a winner's sums over its voxel
	DeviceBuffer owner;                   // uint32 [V]: winning agent per voxel (batches), or the first
										  // slot of the voxel's group in a_sorted (single domain)
	DeviceBuffer counts;                  // uint32 [V]: active agents per voxel

	// measurement
	bool timing = false;
	KernelStat stats[K_COUNT];
	uint64_t launches = 0;
	std::vector<cudaEvent_t> event_pool;
	struct PendingTiming
	{
		int kid;
		cudaEvent_t a, b;
		double per_shared; // algorithmic bytes per agent in a shared voxel (a count known on the device)
		double per_writer; // and per agent that writes a voxel (alone or winner)
	};
	uint32_t shared_agents = 0; // agents in shared voxels after the last timed ballot (timing mode)
	uint32_t writer_agents = 0; // agents that write a voxel after it
	std::vector<PendingTiming> pending;
};

// Launch bookkeeping: every kernel launch goes through begin/end so that the
// context can count launches and (optionally) time them with CUDA events.
void launch_begin(Context* c, int kid, double bytes, cudaEvent_t* ev);
void launch_end(Context* c, int kid, cudaEvent_t ev, double per_shared = 0.0, double per_writer = 0.0);
void collect_timings(Context* c);

// ------------------------------------------------------------------ kernel launchers (defined in .cu files)

int launch_sweep_x(Context* c, bool mass_check = false);
// x and y sweeps of a 3-D mesh fused slab by slab (sweeps.cu), when xy_fusable
bool xy_fusable(const Context* c);
int launch_sweep_xy(Context* c, bool mass_check = false);
int launch_sweep_yz(Context* c, int axis, bool fuse_faces = false, bool mass_check = false);
// Dirichlet faces (unless the last sweep already wrote them) and interior nodes
int launch_dirichlet(Context* c, bool faces_done = false);
// true when the last sweep of c can apply the boundary faces itself
bool faces_fusable(const Context* c);
int launch_bulk(Context* c);
int launch_cells(Context* c, bool recompute);
int launch_release(Context* c, uint64_t agent);
int launch_mass(Context* c, double* dev_out);
// After a checked step's sweeps: the per-substrate masses before and after them
// and the residual into c->mc_out, from the totals the sweeps added to
// c->mc_tot (cleared for the next step).
int launch_mass_check_finish(Context* c);
int launch_to_host_layout(Context* c, void* dst, int layout, int dtype);
int launch_from_host_layout(Context* c, const void* src, int layout, int dtype);
int launch_fill_initial(Context* c); // from the initial values already in c->mass (as T)

// One FP32 cell secretion/uptake pass (ballot rebuilt) over caller-owned device
// buffers, with the scratch arrays supplied by the caller as well; used by the
// allocation-free entry point.
struct CellStepBuffers
{
	int dims;
	uint64_t A, S;
	uint64_t n[3];
	int64_t bbmin[3];
	uint64_t voxel[3];
	uint64_t pitch; // field row pitch (elements)
	double dt;
	const double *pos, *sec, *sat, *upt, *net, *vol;
	const uint8_t* active;
	double* internal;
	int internalized;
	float* field;
	// scratch: vox/foff/shared/rank/role [A], sorted [A] pairs, owner/counts [V], flags/err [4] each,
	// terms [A*S] each
	uint32_t *vox, *foff, *shared, *rank, *owner, *counts, *flags, *err;
	uint2* sorted;
	uint8_t* role;
	float *num, *den, *fac, *rnum, *rden, *rfac;
};
int launch_cells_fp32_buffers(const CellStepBuffers& b, cudaStream_t stream);

// Device bytes a context needs once initialised (admission control).
uint64_t estimate_device_bytes(const Context* c);

// context lifecycle (capi.cu)
int initialize_context(Context* c, bool wait = true); // allocates and uploads on first use
int check_context(Context* c);       // synchronises and reports the device error word
std::string device_error_text(uint32_t word);

struct DeviceGuard
{
	int prev = -1;
	explicit DeviceGuard(int dev)
	{
		cudaGetDevice(&prev);
		if (prev != dev)
			cudaSetDevice(dev);
	}
	~DeviceGuard()
	{
		if (prev >= 0)
			cudaSetDevice(prev);
	}
};

// geometry helpers shared by the launchers and the feasibility checks
uint64_t coef_table_len(uint64_t n, uint64_t S, size_t wsize);
uint64_t coef_row_pitch(uint64_t n);
uint64_t sweep_x_smem_pitch(uint64_t row_len, uint64_t S, size_t wsize);
// x mapping of the single-domain sweep: substrate-per-thread (true) or row-per-thread
bool x_substrate_mapping(uint64_t S);
uint64_t sweep_x_sub_pitch(uint64_t row_len, uint64_t S, size_t wsize);
uint64_t x_threads_per_row(uint64_t S, size_t wsize);
uint64_t sweep_smem_bytes(const Context* c, int axis);
int prepare_sweep_maps(Context* c);
// y/z chunk geometry: points per TMA box and boxes per line
void box_geometry(uint64_t n, uint32_t& box_rows, uint32_t& boxes);
// TMA map of the field as the tensor (x*S+s, y, z) with boxes of box_cols x
// box_rows points along `axis` (1 or 2)
int encode_field_map(const Context* c, int axis, uint32_t box_rows, CUtensorMap* out, uint32_t box_cols = 32);

} // namespace pcg

struct pcg_context : pcg::Context
{};

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

// Returns true when the phase with parity `phase` completed within the time limit.
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

// TMA tile load of a 3-D box at coordinates (c0, c1, c2) into shared memory,
// completing on `bar`; c0 * sizeof(element) must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2,
											uint64_t* bar)
{
	asm volatile(
		"cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
		"[%5];" ::"r"(smem_addr(dst)),
		"l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
		: "memory");
}

// TMA tile store of a 3-D box (elements outside the tensor are not written).
__device__ __forceinline__ void tma_store_3d(const CUtensorMap* map, int c0, int c1, int c2, const void* src)
{
	asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];" ::"l"(map),
				 "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(src))
				 : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Waits until this thread's bulk groups have finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }

// Same, except for the most recently committed group.
__device__ __forceinline__ void bulk_wait_read_allbut1()
{
	asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory");
}

// Waits until this thread's bulk groups have completed.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Makes generic-proxy shared-memory writes visible to the async (bulk copy) proxy.
__device__ __forceinline__ void fence_proxy_async_smem()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ float fmadd(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmadd(double a, double b, double c) { return __fma_rn(a, b, c); }

} // namespace pcg::dev
#endif
