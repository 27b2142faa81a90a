/*
 * physicore_gb300.h -- C ABI of the GB300 BioFVM reaction-diffusion backend.
 *
 * One pcg_context is one BioFVM problem (mesh, substrates, Dirichlet sets, bulk
 * tables, agents) resident on one GPU.  The entry points replace the reference's
 * solver plugin surface, reactions-diffusion/biofvm/include/biofvm/solver.h:12-39,
 * and read the same microenvironment fields the reference solvers read
 * (include/biofvm/microenvironment.h:46-81).  A C++ `solver` subclass that
 * forwards to these calls is in physicore_gb300/csrc/host/gb300_solver.{h,cpp}.
 *
 * Conventions
 *  - Every function returns 0 (PCG_OK) on success or a PCG_ERR_* code; the text
 *    of the last error on the calling thread is returned by pcg_last_error().
 *    The reference reports these conditions with exceptions/asserts
 *    (microenvironment_builder.cpp:153-204, mesh.cpp:39-44).
 *  - Host arrays are plain C arrays; all scalars are double/uint64_t as in the
 *    reference (common/include/common/types.h:7-9).  Nothing is retained: every
 *    setter copies its input.
 *  - Work is queued on the context's CUDA stream; functions that return data to
 *    the host synchronise that stream first.
 *  - Kernels never trap: device-side faults (agent outside the mesh, a bounded
 *    wait that ran out) set a device error word that the next synchronising call
 *    reports as PCG_ERR_DEVICE.
 */
#ifndef PHYSICORE_GB300_H
#define PHYSICORE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PCG_OK 0
#define PCG_ERR_INVALID 1     /* bad argument or call order */
#define PCG_ERR_CUDA 2        /* CUDA runtime error */
#define PCG_ERR_NOMEM 3       /* device or host allocation failed / admission refused */
#define PCG_ERR_DEVICE 4      /* a kernel flagged a fault (see pcg_last_error) */
#define PCG_ERR_UNSUPPORTED 5 /* size beyond the library's limits */

/* Arithmetic of the device field: the reference is FP64 throughout
 * (types.h:7); the FP32 build keeps FP64 coefficients/positions/internalized
 * substrates and stores the substrate field in FP32. */
#define PCG_FP32 0
#define PCG_FP64 1

/* Host buffer layouts for pcg_get_field / pcg_set_field.
 * INTERLEAVED is the reference's layout without row padding
 * (openmp_solver/src/diffusion_solver.h:64-83): index = s + S*(x + nx*(y + ny*z)).
 * PLANAR is substrate-major: index = x + nx*(y + ny*(z + nz*s)). */
#define PCG_LAYOUT_INTERLEAVED 0
#define PCG_LAYOUT_PLANAR 1

/* Host element types for pcg_get_field / pcg_set_field. */
#define PCG_DTYPE_F64 0
#define PCG_DTYPE_F32 1

/* Phases of one step, in the reference's order (openmp_solver.cpp:27-37). */
#define PCG_PHASE_DIFFUSION 1u
#define PCG_PHASE_DIRICHLET 2u
#define PCG_PHASE_BULK 4u
#define PCG_PHASE_CELLS 8u
#define PCG_PHASE_ALL 15u

/* Bulk supply/uptake tables: the reference's virtual bulk_functor
 * (include/biofvm/bulk_functor.h:8-14) evaluated into device tables. */
#define PCG_BULK_NONE 0
#define PCG_BULK_UNIFORM 1   /* supply/uptake/target arrays of length S */
#define PCG_BULK_PER_VOXEL 2 /* arrays of length S*V, planar [s][z][y][x] */

typedef struct pcg_context pcg_context;

/* Per-kernel timing record (pcg_get_kernel_stats). */
typedef struct pcg_kernel_stat
{
	char name[32];
	uint64_t launches;
	double total_ms;          /* CUDA-event time summed over launches (0 when timing is off) */
	double algorithmic_bytes; /* bytes the kernel must move per the roofline model, summed */
} pcg_kernel_stat;

/* ---- lifetime ---------------------------------------------------------- */

/* Creates a context on `device` with its own CUDA stream.  Replaces the
 * registry factory call solver_registry::get (src/solver_registry.cpp:20-29). */
int pcg_create(pcg_context** out, int precision, int device);
/* Releases every device buffer of the context (solver destructor, solver.h:35). */
int pcg_destroy(pcg_context* ctx);
/* Text of the last error raised on this thread ("" when none). */
const char* pcg_last_error(void);
/* Runs later work of this context on `stream` (a cudaStream_t); NULL restores
 * the context's own stream.  The caller keeps `stream` alive while the context
 * uses it (pcg_destroy synchronises the current stream). */
int pcg_set_stream(pcg_context* ctx, void* stream);
int pcg_get_stream(pcg_context* ctx, void** stream);

/* ---- problem description (microenvironment fields) --------------------- */

/* cartesian_mesh(dims, bounding_box_mins, bounding_box_maxs, voxel_shape)
 * (include/biofvm/mesh.h:11-32, src/mesh.cpp:8-28). */
int pcg_set_mesh(pcg_context* ctx, int dims, const int64_t bbox_min[3], const int64_t bbox_max[3],
				 const uint64_t voxel_shape[3]);
int pcg_get_grid(pcg_context* ctx, uint64_t grid_shape[3]);
/* substrates_count, diffusion_timestep, diffusion_coefficients, decay_rates,
 * initial_conditions (microenvironment.h:53-63). */
int pcg_set_substrates(pcg_context* ctx, uint64_t substrates, double dt, const double* diffusion,
					   const double* decay, const double* initial);
/* dirichlet_interior_voxels [K*dims], _values [K*S], _conditions [K*S]
 * (microenvironment.h:65-69).  Re-callable after initialize: this is the upload
 * half of solver::reinitialize_dirichlet (thrust_solver.cpp:61). */
int pcg_set_dirichlet_interior(pcg_context* ctx, uint64_t count, const uint64_t* voxels, const double* values,
							   const uint8_t* conditions);
/* dirichlet_{min,max}_boundary_{values,conditions}[axis] (microenvironment.h:72-75).
 * side 0 = min, 1 = max; values == NULL removes the face. */
int pcg_set_dirichlet_boundary(pcg_context* ctx, int axis, int side, const double* values,
							   const uint8_t* conditions);
/* bulk_fnc (microenvironment.h:78) tabulated; see PCG_BULK_*. */
int pcg_set_bulk(pcg_context* ctx, int mode, const double* supply, const double* uptake, const double* target);
/* Agent SoA (agent_data_generic_storage.h:16-31, base_agent_data_generic_storage.h:66):
 * positions [A*dims], rates [A*S], volumes [A], is_active [A]; internalized and
 * fraction_released may be NULL (zeros).  Marks positional data for recompute. */
int pcg_set_agents(pcg_context* ctx, uint64_t count, const double* positions, const double* secretion,
				   const double* saturation, const double* uptake, const double* net_export, const double* volumes,
				   const uint8_t* is_active, const double* internalized, const double* fraction_released,
				   int compute_internalized);
/* Uploads moved positions and/or activity flags (either may be NULL) of the
 * current agents; the host side of transfer_to_device (data_manager.cpp:61-93). */
int pcg_update_agents(pcg_context* ctx, const double* positions, const uint8_t* is_active);
int pcg_set_internalized(pcg_context* ctx, const double* internalized);

/* ---- the solver plugin surface (solver.h:12-39) ------------------------- */

/* solver::initialize: allocates the field, fills it with the initial
 * conditions, precomputes the Thomas coefficients in FP64
 * (openmp_solver.cpp:8-21, diffusion_solver.cpp:29-113).  Idempotent. */
int pcg_initialize(pcg_context* ctx);
/* Device memory the context will hold once initialised (field, tables, agents and
 * their scratch, transfer staging), for admission control.  Before initialize a
 * context holds no device memory: agents set earlier are staged on the host. */
int pcg_estimate_device_bytes(pcg_context* ctx, uint64_t* bytes);
/* solver::solve(m, iterations) (openmp_solver.cpp:23-40): diffusion x->y->z,
 * Dirichlet, bulk, cells per iteration; ballots are rebuilt during every
 * iteration of a call that follows initialize or pcg_recompute_positional_data. */
int pcg_solve(pcg_context* ctx, uint64_t iterations);
/* Runs the selected phases once (the reference's unit tests drive the
 * sub-solvers this way, e.g. openmp_solver/tests/test_cell_solver.cpp:159-187). */
int pcg_run_phases(pcg_context* ctx, uint32_t phases, int recompute_cells);
/* solver::recompute_positional_data (openmp_solver.cpp:64). */
int pcg_recompute_positional_data(pcg_context* ctx);
/* cell_solver::release_internalized_substrates (cell_solver.cpp:351-374). */
int pcg_release_internalized(pcg_context* ctx, uint64_t agent);

/* ---- host access (get_substrate_density, transfer_to_host) ------------- */

/* Copies the whole field to `host` in the requested layout and element type
 * (transfer_to_host, data_manager.cpp:35-59; get_substrate_density,
 * openmp_solver.cpp:42-56).  Synchronises the stream. */
int pcg_get_field(pcg_context* ctx, void* host, int layout, int dtype);
/* pcg_get_field without waiting: the field is converted on the device, in stream
 * order after the work already enqueued, into one of two staging buffers, and
 * copied to `host` on a copy stream of the context's own, so the copy overlaps the
 * steps enqueued next.  `host` must be pinned (cudaHostAlloc / cudaHostRegister;
 * pageable memory is read back synchronously) and left alone until
 * pcg_wait_field(ticket) returns.  Reserves 2 x V x S x element bytes of device
 * memory at first use. */
int pcg_get_field_async(pcg_context* ctx, void* host, int layout, int dtype, uint64_t* ticket);
/* Waits until the readback `ticket` (and every earlier one) is in host memory. */
int pcg_wait_field(pcg_context* ctx, uint64_t ticket);
/* Overwrites the field from `host` (transfer_to_device of the densities). */
int pcg_set_field(pcg_context* ctx, const void* host, int layout, int dtype);
/* One density, synchronising (the const get_substrate_density). */
int pcg_get_density(pcg_context* ctx, uint64_t s, uint64_t x, uint64_t y, uint64_t z, double* value);
int pcg_get_internalized(pcg_context* ctx, double* host);
/* Active agents per voxel after the last ballot, [V] in x-fastest order.
 * Integer, bit-exact with the reference's ballot (cell_solver.cpp:79-129). */
int pcg_get_counts(pcg_context* ctx, uint32_t* host);
/* 1 when the last ballot found a voxel with more than one agent. */
int pcg_get_conflict(pcg_context* ctx, int* conflict);
/* Total mass per substrate, summed on the device in FP64. */
int pcg_mass(pcg_context* ctx, double* host);

/* Per-step mass conservation check, off by default.  Each sweep matrix has
 * column sums 1 + decay*dt/dims (diffusion_solver.cpp:29-86, the reference's
 * Uniform tests rest on this; an axis of length 1 adds r = dt*D/h^2, its single
 * diagonal entry having r subtracted once), so every step's sweeps must divide
 * each substrate's total by f, the product of those sums over the axes, whatever
 * Dirichlet, bulk and agents then add.  When enabled, every step that runs the diffusion
 * phase totals the field in FP64 before the x sweep and after the last sweep --
 * the sweeps add up the values they read and write, so the check reads no extra
 * pass of the field -- and keeps, per substrate, the worst
 * |after*f - before| / |before|.  Enabling resets the record.  Contexts stepped by
 * a batch keep their check (pcg_batch_solve checks every domain that has it on). */
int pcg_set_mass_check(pcg_context* ctx, int enable);
/* Fusion of the x and y sweeps of 3-D meshes (3 to 32 substrates), off by
 * default: with enable = 1 they run as one launch over z-slabs of about
 * slab_bytes of field, the y sweep of a slab starting at least `lag` slabs after
 * its x sweep, so that the y sweep reads the x sweep's output from L2 (the
 * arithmetic is unchanged; the field crosses HBM four times per step instead of
 * six).  slab_bytes / lag of 0 keep the current values (defaults 8 MiB and 2). */
int pcg_set_sweep_fusion(pcg_context* ctx, int enable, uint64_t slab_bytes, uint32_t lag);
/* The last checked step's totals before and after its sweeps, the worst residual
 * since the check was enabled (each [S], NULL to skip) and the steps checked. */
int pcg_get_mass_check(pcg_context* ctx, double* mass_before, double* mass_after, double* worst_residual,
					   uint64_t* steps_checked);
int pcg_synchronize(pcg_context* ctx);

/* ---- device-resident access (benchmarks, zero-copy integration) -------- */

/* Device pointer of the field, its element size and row pitch (elements).
 * Device layout: the reference's interleaved order with padded rows: element
 * (s,x,y,z) is at ptr[(z*ny + y)*pitch + x*S + s]. */
int pcg_get_field_device(pcg_context* ctx, void** ptr, uint64_t* elem_bytes, uint64_t* pitch);

/* Device pointers of the agents' positions [A*dims] (FP64, agent-major) and
 * activity flags [A] (uint8), for a GPU module that moves agents in place instead
 * of uploading the host SoA every step (the per-step transfers of
 * data_manager.cpp:35-93).  Writes must be ordered before the next step on the
 * context's stream (pcg_get_stream); then pcg_recompute_positional_data, as after
 * pcg_update_agents.  Valid until the agents are set again or the context is
 * destroyed.  Initialises the context if needed. */
int pcg_get_agents_device(pcg_context* ctx, double** positions, uint8_t** is_active);

/* ---- measurement -------------------------------------------------------- */

/* Wraps every kernel launch in CUDA events (per-kernel time) when enabled.  The
 * cell kernels' algorithmic bytes scale with counts known on the device (agents
 * of shared voxels, agents that write a voxel); they are read after every timed
 * ballot, and when timing is enabled after a ballot (this call then waits for
 * the context's stream). */
int pcg_set_kernel_timing(pcg_context* ctx, int enable);
/* Copies up to `cap` per-kernel records; *count receives how many exist. */
int pcg_get_kernel_stats(pcg_context* ctx, pcg_kernel_stat* stats, uint64_t cap, uint64_t* count);
int pcg_reset_kernel_stats(pcg_context* ctx);
/* Kernels launched by this context since creation or the last reset. */
int pcg_get_launch_count(pcg_context* ctx, uint64_t* launches);

/* ---- batches of independent domains -------------------------------------- */

/* No counterpart in the reference, which steps one microenvironment per solver
 * (openmp_solver.cpp:23-40).  A batch steps many initialised contexts of one
 * precision on one device together: every phase of a step is one launch over all
 * domains (one persistent launch per sweep axis, tiles handed out dynamically),
 * and the step is replayed from a CUDA graph.  Each domain's arithmetic and
 * phase order are those of pcg_solve on that context, whose buffers the batch
 * uses in place: results are read back with the per-context calls.
 *  - The contexts stay owned by the caller and must outlive the batch; setters
 *    that change a context's sizes or tables are picked up at the next
 *    pcg_batch_solve (descriptors rebuilt, graph re-captured).
 *  - Work is queued on the batch's stream, ordered after each context's stream
 *    on entry and before it on return, so per-context calls see the results. */
typedef struct pcg_batch pcg_batch;

int pcg_batch_create(pcg_batch** out, pcg_context* const* contexts, uint64_t count);
int pcg_batch_destroy(pcg_batch* batch);
/* `iterations` steps of every domain (solver::solve; a context whose positional
 * data are marked for recomputation rebuilds its ballot on each of them). */
int pcg_batch_solve(pcg_batch* batch, uint64_t iterations);
/* `iterations` steps in which domain d takes part in the first budgets[d] only
 * (0: it sits this call out); lets requests of different lengths share launches
 * and finish inside one call. */
int pcg_batch_solve_budgets(pcg_batch* batch, uint64_t iterations, const uint64_t* budgets);
int pcg_batch_synchronize(pcg_batch* batch);
int pcg_batch_get_stream(pcg_batch* batch, void** stream);
/* Replays the step from a CUDA graph (default 1) or launches it directly. */
int pcg_batch_set_graph(pcg_batch* batch, int enable);
/* Builds the descriptors and captures both step graphs (with and without the
 * ballot-rebuild kernels) now, without running anything, so that the first solve
 * launches at once.  It touches only the batch's own buffers and stream: a batch
 * can be prepared while another batch over the same contexts is stepping them. */
int pcg_batch_prepare(pcg_batch* batch);
/* Times candidate line mappings and tile shapes of each sweep axis for each size
 * bucket (line length, substrates) present in the batch and keeps the fastest;
 * results are cached for the process.  Field contents are restored afterwards. */
int pcg_batch_autotune(pcg_batch* batch);
/* Overrides the autotuner for one sweep axis of every domain (tests, experiments).
 * x: mapping PCG_MAP_ROW (a thread owns a row) or PCG_MAP_SUBSTRATE (a thread owns
 * one substrate of a row); y/z: PCG_MAP_COLUMN (a lane owns one (x,s) column).
 * rows = rows per x tile or points per y/z TMA box (0: the default), clamped per
 * domain to what fits.  mapping < 0 removes the override. */
#define PCG_MAP_ROW 0
#define PCG_MAP_SUBSTRATE 1
#define PCG_MAP_COLUMN 0
int pcg_batch_force_config(pcg_batch* batch, int axis, int mapping, uint32_t rows);
/* Writes a JSON description of the per-bucket choices (NUL-terminated, at most
 * cap bytes); *needed receives the full length including the NUL. */
int pcg_batch_describe(pcg_batch* batch, char* text, uint64_t cap, uint64_t* needed);
int pcg_batch_set_kernel_timing(pcg_batch* batch, int enable);
int pcg_batch_get_kernel_stats(pcg_batch* batch, pcg_kernel_stat* stats, uint64_t cap, uint64_t* count);
int pcg_batch_reset_kernel_stats(pcg_batch* batch);
/* Kernels launched by this batch (graph replays count their kernels). */
int pcg_batch_get_launch_count(pcg_batch* batch, uint64_t* launches);

/* ---- serving: continuous batching of independent simulations ------------- */

/* No counterpart in the reference, which runs one simulation per process.  A
 * server owns a worker thread that admits requests by free device memory, keeps
 * them resident, steps all admitted ones together through one batch (regrouped
 * between ticks as requests finish and arrive), and hands finished ones back.
 *  - A request is a context configured with the setters but NOT initialised (it
 *    holds no device memory yet: agents set before initialize are staged on the
 *    host); the server initialises it on admission.  From submit until it comes
 *    back from pcg_server_poll the server owns it: do not call into it meanwhile.
 *  - A returned context holds its results (read them with pcg_get_field etc.)
 *    and its device memory until the caller destroys it, so poll and destroy
 *    promptly: the memory of finished requests is what later admissions use.
 *  - Admission: requests are taken in arrival order while the next one's device
 *    bytes (pcg_estimate_device_bytes) plus reserve_bytes fit in free memory;
 *    while active requests hold memory a request waits; one that cannot fit with
 *    nothing active is refused.  memory_limit_bytes (0: the device's free memory)
 *    caps the memory the server may use. */
typedef struct pcg_server pcg_server;

typedef struct pcg_server_options
{
	uint64_t max_active;         /* simulations stepped together (0: 1024) */
	uint64_t steps_per_tick;     /* steps between admission points (0: 8) */
	uint64_t reserve_bytes;      /* free memory kept back at admission */
	uint64_t max_queue;          /* queued requests before submissions are refused (0: 2^20) */
	uint64_t memory_limit_bytes; /* 0: use the device's free memory */
	int autotune;                /* autotune new size buckets when the batch is regrouped */
} pcg_server_options;

#define PCG_REQUEST_DONE 0
#define PCG_REQUEST_CANCELLED 1
#define PCG_REQUEST_REFUSED 2
#define PCG_REQUEST_FAILED 3

typedef struct pcg_server_result
{
	pcg_context* ctx;
	uint64_t tag;
	uint64_t steps;
	int status;               /* PCG_REQUEST_* */
	int code;                 /* PCG_ERR_* behind a refusal or failure */
	double t_submit, t_admit, t_done; /* seconds since the server started; t_admit < 0: never admitted */
	uint64_t device_bytes;    /* estimate used for admission */
	char error[160];
} pcg_server_result;

typedef struct pcg_server_stats
{
	uint64_t submitted, admitted, completed, cancelled, refused, failed;
	uint64_t ticks, rebuilds, steps;
	uint64_t vss;            /* voxel-substrate-steps performed */
	uint64_t active_bytes;   /* device bytes of the admitted set */
	uint64_t queued, active, in_flight;
	double uptime_s;
	/* worker time regrouping the active set into a batch, starting and waiting
	 * for steps, and admitting requests */
	double rebuild_s, step_s, admit_s;
	/* next-tick batches built (and their graphs captured) while a tick's steps
	 * ran, and the worker time spent on them; a tick whose set matches its
	 * prepared batch starts without a rebuild */
	uint64_t prebuilds;
	double prebuild_s;
} pcg_server_stats;

int pcg_server_create(pcg_server** out, int precision, int device, const pcg_server_options* options);
/* Stops the worker; contexts the server still holds are destroyed. */
int pcg_server_destroy(pcg_server* server);
int pcg_server_submit(pcg_server* server, pcg_context* request, uint64_t steps, uint64_t tag);
/* pcg_server_submit, and when the request is done the server copies its field
 * into `host` (layouts and types as pcg_get_field; pinned memory recommended)
 * right after the steps in which it finished, before reporting it: the copies of
 * finished requests then run while the device has no other work of the server,
 * and the caller's thread issues no device work of its own.  `host` must stay
 * valid until the request is returned by pcg_server_poll. */
int pcg_server_submit_readback(pcg_server* server, pcg_context* request, uint64_t steps, uint64_t tag, void* host,
							   int layout, int dtype);
/* Cancels a queued or running request (it comes back with PCG_REQUEST_CANCELLED). */
int pcg_server_cancel(pcg_server* server, uint64_t tag);
/* Up to `cap` finished requests; waits up to wait_ms for the first. */
int pcg_server_poll(pcg_server* server, pcg_server_result* results, uint64_t cap, uint64_t* count, int wait_ms);
int pcg_server_get_stats(pcg_server* server, pcg_server_stats* stats);

/* ---- allocation-free cell step ------------------------------------------- */

/* No counterpart in the reference.  For callers that cannot let a library
 * allocate device memory -- frameworks that serve all GPU memory from their own
 * pool or arena, and loops that must avoid the device synchronisation of
 * cudaMalloc/cudaFree -- this runs one cell secretion/uptake pass (ballot rebuilt,
 * then the density and internalized updates; cell_solver.cpp:246-272 with
 * recompute) on buffers the caller owns, and allocates nothing.
 *
 *  - field: FP32 device field in the interleaved layout with row pitch `pitch`
 *    elements (>= grid_shape[0] * substrates), rows ordered by y then z.
 *  - All agent arrays are device pointers, laid out as in pcg_set_agents;
 *    internalized is updated in place when compute_internalized is non-zero.
 *  - Work is queued on `stream` (NULL: the default stream); every call then
 *    copies the device error word to the host and synchronises that stream to
 *    report device faults (PCG_ERR_DEVICE), so the call blocks until its work is
 *    done and cannot be recorded into a CUDA graph by stream capture.
 *  - Scratch comes from one fixed 16 MiB array in device memory that every GPU
 *    loading this library holds until the process exits; a problem that needs
 *    more (about 8 bytes per voxel plus 25 + 24*substrates bytes per agent) is
 *    rejected with PCG_ERR_UNSUPPORTED, as are meshes of 2^32 - 1 or more voxels,
 *    2^32 - 1 or more agents and fields of 2^32 or more elements (pitch * ny *
 *    nz).  grid_shape must be 1 on the axes beyond dims (PCG_ERR_INVALID).  The
 *    first call on a device looks up the array's device address.
 *  - All calls share the array, which keeps the last call's contents: calls that
 *    overlap on the GPU (other streams, other host threads) race with each other
 *    and must be serialised by the caller. */
int pcg_cells_noalloc(float* field, uint64_t pitch, int dims, const int64_t bbox_min[3],
					  const uint64_t voxel_shape[3], const uint64_t grid_shape[3], uint64_t substrates, double dt,
					  uint64_t agents, const double* positions, const double* secretion, const double* saturation,
					  const double* uptake, const double* net_export, const double* volumes, const uint8_t* is_active,
					  double* internalized, int compute_internalized, void* stream);

#ifdef __cplusplus
}
#endif

#endif
