// sweeps.cu -- ADI/LOD Thomas sweeps along x, y and z on sm_103a.
//
// Arithmetic per line follows the reference (openmp_solver/src/diffusion_solver.cpp:
// 116-202 for x, 390-794 for y/z; coefficients of diffusion_solver.cpp:29-86):
//   forward   d_i  = d_i + e_{i-1} d_{i-1}            i = 1..n-1
//             d_{n-1} = d_{n-1} b'_{n-1}
//   backward  d_i  = (d_i + c d_{i+1}) b'_i            i = n-2..0
// with each line using the coefficients of its own substrate.  Both passes start
// from a zero carry: e_{-1} = 0 makes the first forward step d_0 = d_0, and c*0 = 0
// makes the first backward step d_{n-1} b'_{n-1}, so every step has one form.
//
// GB300 mapping (our own design):
//  * A line must stay on chip between its forward and backward pass, so shared
//    memory bounds how many lines an SM can hold (~160 lines of 320 FP32 points).
//    Every byte of it therefore holds line data: tiles are single-stage, the
//    coefficient tables are read through L1 (__ldg, 16-byte vectors), and tile
//    sizes are chosen so that several CTAs share an SM and all four schedulers
//    have warps to issue.
//  * Persistent CTAs (one warp) walk their tiles: TMA loads complete on an
//    mbarrier, the warp solves the tile in place, and TMA stores write it back; the
//    next load is issued as soon as the stores have read shared memory.  Several
//    such CTAs per SM overlap one another's loads, compute and stores.
//  * Solvers run in blocks of P steps without per-step predicates; the next block's
//    points and coefficients are requested before the current block's dependent
//    chain, so load latency overlaps the chain.
//  * y/z: a tile is 32 consecutive (x,s) elements of a row at every point of the
//    lines; lane t solves column t of the [n][32] tile (bank-conflict free) with
//    the coefficient row of its substrate ([s][j] table).
//  * x: a tile is R whole rows; a row is walked as a stream of 16-byte chunks,
//    element k belonging to substrate k % S, with one carry per substrate.  When a
//    voxel's substrates fill whole chunks, TPR threads share a row, one chunk slot
//    each; rows are TPR (mod 8) chunks apart so quarter-warps hit distinct banks.
//  * Every wait is bounded; a timeout sets a device error bit instead of trapping.
#include "field_device.cuh"
#include "pcg_internal.cuh"
#include "sweep_solvers.cuh"

namespace pcg {

namespace {

using namespace solvers;

// ------------------------------------------------------------------ y / z

// The y/z sweep.  A tile is 32 consecutive (x,s) elements at all n points of the
// lines of one outer index; it arrives as nc TMA tensor boxes (32, R) of the field
// described as the 3-D tensor (x*S+s, y, z), all completing on one mbarrier.  The
// warp solves the tile in place and stores it back with nc box stores; the next
// tile's loads start once the stores have read shared memory.  Loads and compute
// overlap across the several single-warp CTAs an SM holds; within a CTA the solver
// runs without per-chunk bookkeeping.  Coefficients come from the compressed
// tables (head rows, then per-substrate constants), so most points need no
// coefficient load at all.
//
// MC = kMcOut (the step's last sweep with the mass check on): the lanes also sum
// their solved values before the faces are written, into a.mc_tot[S + s].  A
// lane's substrate is the same in every tile when S divides 32 (it then keeps one
// running total and adds it once at the end), else it adds its total per tile.
template <typename T, int AXIS, int MC>
__global__ void __launch_bounds__(kLanes) sweep_yz_kernel(SweepArgs a, const __grid_constant__ CUtensorMap tmap)
{
	extern __shared__ __align__(128) unsigned char smem[];
	uint64_t* full = reinterpret_cast<uint64_t*>(smem);
	T* base = reinterpret_cast<T*>(smem + 128);
	const uint32_t lane = threadIdx.x;
	const uint32_t n = a.n, S = a.S, R = a.box_rows, nc = a.boxes;
	const uint32_t chunk_elems = R * kLanes;
	const T* comp = static_cast<const T*>(a.coef) + a.comp_off;
	if (lane == 0)
	{
		dev::mbar_init(full, 1);
		dev::fence_mbar_init();
	}
	__syncwarp();
	bool ok = true;
	MassAcc<T> acc;
	acc.zero();
	const bool per_tile = (kLanes % S) != 0;
	const uint32_t classes = S < kLanes ? S : kLanes;
	// 32-bit tile arithmetic: a launch has fewer than 2^32 tiles
	const uint32_t xblocks = (uint32_t)a.xblocks, nouter = (uint32_t)(a.tiles / a.xblocks);
	for (uint32_t phase = 0;; phase ^= 1)
	{
		uint32_t t32 = 0;
		if (lane == 0)
			t32 = atomicAdd(a.ticket, 1u);
		const uint32_t t = __shfl_sync(0xffffffffu, t32, 0);
		if (t >= a.tiles)
			break;
		const int x0 = (int)((t % xblocks) * kLanes);
		// y takes its z-planes from the last down: the x sweep that ran just before
		// wrote the highest planes last, and their lines are still in L2
		const int o = AXIS == 1 ? (int)(nouter - 1 - t / xblocks) : (int)(t / xblocks);
		if (lane == 0)
		{
			dev::mbar_arrive_expect_tx(full, nc * chunk_elems * (uint32_t)sizeof(T));
			for (uint32_t c = 0; c < nc; c++)
			{
				if (AXIS == 1)
					dev::tma_load_3d(base + c * chunk_elems, &tmap, x0, (int)(c * R), o, full);
				else
					dev::tma_load_3d(base + c * chunk_elems, &tmap, x0, o, (int)(c * R), full);
			}
		}
		// lanes past the row hold zero-filled columns that are never stored
		const uint32_t s = (uint64_t)(x0 + lane) < a.row_len ? (uint32_t)((x0 + lane) % S) : 0;
		const LineCoef<T> L = line_coef<T>(comp, S, a.head, n, s);
		ok = __all_sync(0xffffffffu, dev::mbar_wait(full, phase));
		if (!ok)
			break;
		solve_line<T, kLanes, MC>(base + lane, n, 0, L, nullptr, &acc);
		if constexpr ((MC & kMcOut) != 0)
			if (per_tile)
			{
				flush_classes(acc.value(), classes, kLanes, a.mc_tot + S + ((uint64_t)x0 + lane) % S);
				acc.zero();
			}
		if (a.face_mask)
		{
			FaceArgs f {};
			f.values = a.face_values;
			f.conds = a.face_conds;
			f.face_mask = a.face_mask;
			f.S = S;
			f.nx = a.nx, f.ny = a.ny, f.nz = a.nz;
			fielddev::faces_on_column<T, AXIS>(f, base + lane, n, kLanes, (uint64_t)x0 + lane, (uint64_t)o);
		}
		dev::fence_proxy_async_smem();
		__syncwarp();
		if (lane == 0)
		{
			for (uint32_t c = 0; c < nc; c++)
			{
				if (AXIS == 1)
					dev::tma_store_3d(&tmap, x0, (int)(c * R), o, base + c * chunk_elems);
				else
					dev::tma_store_3d(&tmap, x0, o, (int)(c * R), base + c * chunk_elems);
			}
			dev::bulk_commit();
			dev::bulk_wait_read();
		}
		__syncwarp();
	}
	if constexpr ((MC & kMcOut) != 0)
		if (!per_tile)
			flush_classes(acc.value(), classes, kLanes, a.mc_tot + S + lane % S);
	if (!ok && lane == 0)
		atomicOr(a.err, DEV_ERR_WAIT_TIMEOUT);
	if (lane == 0)
		dev::bulk_wait_all();
}

// ------------------------------------------------------------------ x

// Row-per-thread mapping: a tile is rows_per_tile consecutive rows and the CTA has
// rows_per_tile * TPR threads (<= 32); TPR threads share a row when its substrates
// fill whole 16-byte chunks.
// MC (the mass check on): the threads also sum their rows' inputs (kMcIn) and, on
// a 1-D mesh where x is the last sweep, their outputs (kMcOut) per substrate.
template <typename T, int ST, int MC>
__global__ void __launch_bounds__(kLanes) sweep_x_kernel(SweepArgs a)
{
	constexpr int TPR = x_tpr<T, ST>();
	constexpr bool kChunks = ST > 0 && (ST * (int)sizeof(T)) % 16 == 0;
	constexpr int NA = kChunks ? Vec16<T>::N : (ST > 0 ? ST : 1);
	MassAcc<T> ai[NA], ao[NA];
#pragma unroll
	for (int u = 0; u < NA; u++)
	{
		ai[u].zero();
		ao[u].zero();
	}
	extern __shared__ __align__(128) unsigned char smem[];
	uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
	uint32_t& ticket = *reinterpret_cast<uint32_t*>(smem + 8);
	T* tile = reinterpret_cast<T*>(smem + 16);
	const int tid = threadIdx.x;
	const uint32_t R = a.rows_per_tile;
	const int r_local = tid / TPR, h = tid % TPR;
	const uint32_t n = a.n;
	const uint32_t row_bytes = (uint32_t)round_up(a.row_len * sizeof(T), 16);
	const T* cB = static_cast<const T*>(a.coef);
	const T* cE = cB + a.coef_len;
	const T* cC = cE + a.coef_len;
	const T* cBl = sizeof(T) == 4 ? cB + a.blo_off : nullptr;
	if (tid == 0)
	{
		dev::mbar_init(bar, 1);
		dev::fence_mbar_init();
	}
	__syncthreads();

	for (uint32_t phase = 0;; phase ^= 1)
	{
		if (tid == 0)
			ticket = atomicAdd(a.ticket, 1u);
		__syncthreads();
		const uint64_t t = ticket;
		if (t >= a.tiles)
			break;
		const uint64_t r0 = t * R;
		const uint32_t nrows = (uint32_t)(a.rows - r0 < (uint64_t)R ? a.rows - r0 : (uint64_t)R);
		T* g = static_cast<T*>(a.field) + r0 * a.pitch;
		if (tid == 0)
			dev::mbar_arrive_expect_tx(bar, nrows * row_bytes);
		__syncthreads();
		if ((uint32_t)tid < nrows)
			dev::bulk_g2s(tile + tid * a.smem_pitch, g + tid * a.pitch, row_bytes, bar);
		if (!__syncthreads_and(dev::mbar_wait(bar, phase)))
		{
			if (tid == 0)
				atomicOr(a.err, DEV_ERR_WAIT_TIMEOUT);
			break;
		}
		if ((uint32_t)r_local < nrows)
		{
			T* row = tile + r_local * a.smem_pitch;
			if constexpr (ST == 0)
				solve_row_generic<T, MC>(row, cB, cE, cC, cBl, n, a.S, a.mc_tot, a.mc_tot + a.S);
			else if constexpr (kChunks)
				solve_row_chunks<T, TPR, MC>(row, cB, cE, cC, cBl, n, h, ai, ao);
			else
				solve_row_vec<T, ST, MC>(row, cB, cE, cC, cBl, n, ai, ao);
		}
		dev::fence_proxy_async_smem();
		__syncthreads();
		if ((uint32_t)tid < nrows)
			dev::bulk_s2g(g + tid * a.pitch, tile + tid * a.smem_pitch, row_bytes);
		dev::bulk_commit();
		dev::bulk_wait_read();
		__syncthreads();
	}
	if constexpr (MC != 0 && ST > 0)
	{
		// thread r * TPR + h holds substrates h * VN + u (chunks) or u (one thread per row)
#pragma unroll
		for (int u = 0; u < NA; u++)
		{
			const uint32_t sub = kChunks ? (uint32_t)(h * Vec16<T>::N + u) : (uint32_t)u;
			flush_classes(ai[u].value(), TPR, blockDim.x, a.mc_tot + sub);
			if constexpr ((MC & kMcOut) != 0)
				flush_classes(ao[u].value(), TPR, blockDim.x, a.mc_tot + a.S + sub);
		}
	}
	dev::bulk_wait_all();
}

// Substrate-per-thread mapping: a tile is rows_per_tile rows and thread
// (r, s) = (tid / S, tid % S) solves substrate s of row r, a line of n points
// S elements apart in shared memory, with the compressed coefficients of s (most
// points need no coefficient load).  Row pitches are chosen so that the lanes of
// a warp touch distinct banks.
// ST = S when it is a compile-time constant (stride-S shared-memory accesses with
// immediate offsets), 0 for the run-time path.  MC (the mass check on): lane
// (r, s) also sums its lines' inputs (kMcIn) and, on a 1-D mesh, outputs (kMcOut)
// over all its tiles, added once at the end.
template <typename T, int ST, int MC>
__global__ void __launch_bounds__(kLanes) sweep_x_sub_kernel(SweepArgs a)
{
	extern __shared__ __align__(128) unsigned char smem[];
	uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
	uint32_t& ticket = *reinterpret_cast<uint32_t*>(smem + 8);
	T* tile = reinterpret_cast<T*>(smem + 16);
	const uint32_t tid = threadIdx.x;
	const uint32_t R = a.rows_per_tile, S = ST ? (uint32_t)ST : a.S, n = a.n;
	const uint32_t r_local = tid / S, s = tid % S;
	const uint32_t row_bytes = (uint32_t)round_up(a.row_len * sizeof(T), 16);
	const LineCoef<T> L = line_coef<T>(static_cast<const T*>(a.coef) + a.comp_off, S, a.head, n, s);
	MassAcc<T> ai, ao;
	ai.zero();
	ao.zero();
	if (tid == 0)
	{
		dev::mbar_init(bar, 1);
		dev::fence_mbar_init();
	}
	__syncthreads();
	for (uint32_t phase = 0;; phase ^= 1)
	{
		if (tid == 0)
			ticket = atomicAdd(a.ticket, 1u);
		__syncthreads();
		const uint64_t t = ticket;
		if (t >= a.tiles)
			break;
		const uint64_t r0 = t * R;
		const uint32_t nrows = (uint32_t)(a.rows - r0 < (uint64_t)R ? a.rows - r0 : (uint64_t)R);
		T* g = static_cast<T*>(a.field) + r0 * a.pitch;
		if (tid == 0)
			dev::mbar_arrive_expect_tx(bar, nrows * row_bytes);
		__syncthreads();
		if (tid < nrows)
			dev::bulk_g2s(tile + tid * a.smem_pitch, g + tid * a.pitch, row_bytes, bar);
		if (!__syncthreads_and(dev::mbar_wait(bar, phase)))
		{
			if (tid == 0)
				atomicOr(a.err, DEV_ERR_WAIT_TIMEOUT);
			break;
		}
		if (r_local < nrows)
			solve_line<T, ST, MC>(tile + r_local * a.smem_pitch + s, n, S, L, &ai, &ao);
		dev::fence_proxy_async_smem();
		__syncthreads();
		if (tid < nrows)
			dev::bulk_s2g(g + tid * a.pitch, tile + tid * a.smem_pitch, row_bytes);
		dev::bulk_commit();
		dev::bulk_wait_read();
		__syncthreads();
	}
	if constexpr (MC != 0)
	{
		// lanes r * S + s share substrate s (S <= 32 on this mapping)
		flush_classes(ai.value(), S, kLanes, a.mc_tot + s);
		if constexpr ((MC & kMcOut) != 0)
			flush_classes(ao.value(), S, kLanes, a.mc_tot + S + s);
	}
	dev::bulk_wait_all();
}

// ------------------------------------------------------------------ fused x + y

// The x and y sweeps of a 3-D mesh in one persistent launch, z-slab by z-slab.
// x lines and y lines of a z-plane both lie in that plane, so once the x sweep
// has written the planes of a slab, the y sweep of that slab can start -- while
// the x output is still in L2 (the slabs are a few MB and the y sweep reads
// them a slab or two later).  The y tiles then load from L2 instead of HBM and
// the x output is overwritten in L2 before most of it is ever written back: per
// step the field crosses HBM four times instead of six.  The arithmetic of each
// line is unchanged.
//
// Work items are tickets over a table of segments in ticket order: the x tiles
// of slab k (segment X(k)), and the y tiles of slab k - L after X(k) (lag L).
// A y tile waits until every x tile of its slab has signalled (a per-slab
// counter, released by an x tile after its stores completed and acquired by the
// y tile before its tensor loads).  Tickets are handed out in order and an x
// tile never waits, so every awaited x tile belongs to a running CTA and every
// wait ends; the wait is bounded all the same (DEV_ERR_WAIT_TIMEOUT).  An x tile
// signals once the next tile's loads are in flight (its stores had that long to
// land), and before its CTA waits for any slab.
struct XYArgs
{
	const uint4* segs; // {first ticket, slab | kYSeg, tiles, x tiles of the slab (y segments)}
	uint32_t nseg;
	uint32_t total;    // tickets
	uint32_t planes;   // z-planes per slab
	uint32_t* done;    // [slabs] x tiles signalled, zeroed before the launch
	uint32_t* ticket;
	uint64_t ny, nz;
};
constexpr uint32_t kYSeg = 0x80000000u;

__device__ __forceinline__ uint32_t load_acquire(const uint32_t* p)
{
	uint32_t v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ void fence_proxy_async_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }

// Bounded wait for *p >= target (the calling lane only).
__device__ __forceinline__ bool wait_at_least(const uint32_t* p, uint32_t target)
{
	const uint64_t t0 = dev::global_ns();
	while (load_acquire(p) < target)
	{
		if (dev::global_ns() - t0 > dev::kWaitNs)
			return false;
		__nanosleep(100);
	}
	return true;
}

template <typename T, int ST, int MC>
__global__ void __launch_bounds__(kLanes)
	sweep_xy_kernel(SweepArgs ax, SweepArgs ay, const __grid_constant__ CUtensorMap tmap, XYArgs f)
{
	extern __shared__ __align__(128) unsigned char smem[];
	uint64_t* bar_x = reinterpret_cast<uint64_t*>(smem);
	uint64_t* bar_y = reinterpret_cast<uint64_t*>(smem + 8);
	uint32_t* s_ticket = reinterpret_cast<uint32_t*>(smem + 16);
	T* buf = reinterpret_cast<T*>(smem + 128);
	const uint32_t tid = threadIdx.x;
	// x: lane (r, s) solves substrate s of row r of the tile
	const uint32_t S = ST ? (uint32_t)ST : ax.S, nx_pts = ax.n, R = ax.rows_per_tile;
	const uint32_t r_local = tid / S, s = tid % S;
	const uint32_t row_bytes = (uint32_t)round_up(ax.row_len * sizeof(T), 16);
	const LineCoef<T> Lx = line_coef<T>(static_cast<const T*>(ax.coef) + ax.comp_off, S, ax.head, nx_pts, s);
	MassAcc<T> ai, ao;
	ai.zero();
	ao.zero();
	// y
	const uint32_t ny_pts = ay.n, Ry = ay.box_rows, nc = ay.boxes, chunk_elems = Ry * kLanes;
	const T* ycomp = static_cast<const T*>(ay.coef) + ay.comp_off;
	if (tid == 0)
	{
		dev::mbar_init(bar_x, 1);
		dev::mbar_init(bar_y, 1);
		dev::fence_mbar_init();
	}
	__syncthreads();
	uint32_t phase_x = 0, phase_y = 0;
	int pending = -1; // slab of this CTA's last x tile, not yet signalled
	bool ok = true;
	// signals the pending x tile once its stores have completed
	auto signal = [&]() {
		if (pending < 0)
			return;
		dev::bulk_wait_all();
		fence_proxy_async_global();
		__syncthreads();
		if (tid == 0)
		{
			__threadfence();
			atomicAdd(f.done + pending, 1u);
		}
		pending = -1;
	};
	for (;;)
	{
		if (tid == 0)
			*s_ticket = atomicAdd(f.ticket, 1u);
		__syncthreads();
		const uint32_t t = *s_ticket;
		__syncthreads();
		if (t >= f.total)
			break;
		// the segment holding t (segments are in ticket order)
		uint32_t lo = 0, hi = f.nseg;
		while (hi - lo > 1)
		{
			const uint32_t mid = (lo + hi) / 2;
			if (__ldg(&f.segs[mid].x) <= t)
				lo = mid;
			else
				hi = mid;
		}
		const uint4 seg = __ldg(f.segs + lo);
		const uint32_t u = t - seg.x, slab = seg.y & ~kYSeg;
		if (!(seg.y & kYSeg))
		{
			// x tile u of the slab: rows [r0, r0 + nrows)
			const uint64_t slab_r0 = (uint64_t)slab * f.planes * f.ny;
			const uint64_t slab_r1 = min((uint64_t)(slab + 1) * f.planes, f.nz) * f.ny;
			const uint64_t r0 = slab_r0 + (uint64_t)u * R;
			const uint32_t nrows = (uint32_t)min((uint64_t)R, slab_r1 - r0);
			T* g = static_cast<T*>(ax.field) + r0 * ax.pitch;
			if (tid == 0)
				dev::mbar_arrive_expect_tx(bar_x, nrows * row_bytes);
			__syncthreads();
			if (tid < nrows)
				dev::bulk_g2s(buf + tid * ax.smem_pitch, g + tid * ax.pitch, row_bytes, bar_x);
			signal(); // the previous x tile's stores had this long to complete
			if (!__syncthreads_and(dev::mbar_wait(bar_x, phase_x)))
			{
				ok = false;
				break;
			}
			phase_x ^= 1;
			if (r_local < nrows)
				solve_line<T, ST, MC>(buf + r_local * ax.smem_pitch + s, nx_pts, S, Lx, &ai, &ao);
			dev::fence_proxy_async_smem();
			__syncthreads();
			if (tid < nrows)
				dev::bulk_s2g(g + tid * ax.pitch, buf + tid * ax.smem_pitch, row_bytes);
			dev::bulk_commit();
			dev::bulk_wait_read();
			__syncthreads();
			pending = (int)slab;
		}
		else
		{
			signal(); // never wait on a slab while holding an unsignalled x tile
			bool ready = true;
			if (tid == 0)
			{
				ready = wait_at_least(f.done + slab, seg.w);
				fence_proxy_async_global(); // the tensor loads below follow the acquire
			}
			if (!__syncthreads_and(ready))
			{
				ok = false;
				break;
			}
			// y tile u of the slab: 32 columns at every y of one plane
			const uint32_t xblocks = (uint32_t)ay.xblocks;
			const int x0 = (int)((u % xblocks) * kLanes);
			const int o = (int)((uint64_t)slab * f.planes + u / xblocks);
			if (tid == 0)
			{
				dev::mbar_arrive_expect_tx(bar_y, nc * chunk_elems * (uint32_t)sizeof(T));
				for (uint32_t c = 0; c < nc; c++)
					dev::tma_load_3d(buf + c * chunk_elems, &tmap, x0, (int)(c * Ry), o, bar_y);
			}
			const uint32_t sy = (uint64_t)(x0 + tid) < ay.row_len ? (uint32_t)((x0 + tid) % ay.S) : 0;
			const LineCoef<T> Ly = line_coef<T>(ycomp, ay.S, ay.head, ny_pts, sy);
			if (!__all_sync(0xffffffffu, dev::mbar_wait(bar_y, phase_y)))
			{
				ok = false;
				break;
			}
			phase_y ^= 1;
			solve_line<T, kLanes>(buf + tid, ny_pts, 0, Ly);
			dev::fence_proxy_async_smem();
			__syncwarp();
			if (tid == 0)
			{
				for (uint32_t c = 0; c < nc; c++)
					dev::tma_store_3d(&tmap, x0, (int)(c * Ry), o, buf + c * chunk_elems);
				dev::bulk_commit();
				dev::bulk_wait_read();
			}
			__syncthreads();
		}
	}
	signal();
	if (!ok && tid == 0)
		atomicOr(ax.err, DEV_ERR_WAIT_TIMEOUT);
	if constexpr (MC != 0)
		flush_classes(ai.value(), S, kLanes, ax.mc_tot + s);
	dev::bulk_wait_all();
}

struct Plan
{
	uint64_t smem;
	int threads;
	uint64_t rows_per_tile;
};

template <typename T>
Plan plan(const Context* c, int axis)
{
	Plan p {};
	if (axis == 0 && x_substrate_mapping(c->S))
	{
		const uint64_t row_stage = sweep_x_sub_pitch(c->row_len, c->S, sizeof(T)) * sizeof(T);
		// ~32 KB tiles: more CTAs (warps) per SM beat fuller warps here
		uint64_t rows = std::min<uint64_t>(kXTileBytes / row_stage, kLanes / c->S);
		rows = std::max<uint64_t>(rows, 1);
		p.rows_per_tile = rows;
		p.smem = 16 + rows * row_stage;
		p.threads = kLanes; // lanes past rows * S idle
		return p;
	}
	if (axis == 0)
	{
		const uint64_t row_stage = sweep_x_smem_pitch(c->row_len, c->S, sizeof(T)) * sizeof(T);
		const uint64_t tpr = x_threads_per_row(c->S, sizeof(T));
		// aim for >= 4 CTAs per SM so that every scheduler has a warp
		uint64_t rows = (kMaxSmemBytes / 4) / row_stage;
		const uint64_t cap = kLanes / tpr;
		rows = rows < 1 ? 1 : (rows > cap ? cap : rows);
		p.rows_per_tile = rows;
		p.smem = 16 + rows * row_stage;
		p.threads = (int)(rows * tpr);
		return p;
	}
	uint32_t box_rows, boxes;
	box_geometry(c->n[axis], box_rows, boxes);
	p.smem = 128 + (uint64_t)boxes * box_rows * kLanes * sizeof(T);
	p.threads = kLanes;
	return p;
}

template <typename KernelT>
int launch_persistent(Context* c, KernelT kernel, const SweepArgs& a, const Plan& p, int kid, double bytes)
{
	PCG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem));
	int per_sm = 0;
	PCG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, p.threads, p.smem));
	if (per_sm < 1)
		return fail(PCG_ERR_UNSUPPORTED, "sweep tile does not fit in shared memory");
	uint64_t grid = (uint64_t)per_sm * (uint64_t)c->sm_count;
	if (grid > a.tiles)
		grid = a.tiles;
	PCG_CUDA_TRY(cudaMemsetAsync(a.ticket, 0, sizeof(uint32_t), c->stream));
	cudaEvent_t ev;
	launch_begin(c, kid, bytes, &ev);
	kernel<<<(unsigned)grid, p.threads, p.smem, c->stream>>>(a);
	launch_end(c, kid, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

SweepArgs base_args(const Context* c, int axis)
{
	SweepArgs a {};
	a.field = c->field.ptr;
	a.coef = c->coef[axis].ptr;
	a.coef_len = c->coef_len[axis];
	a.coef_elems = c->coef_elems[axis];
	a.S = (uint32_t)c->S;
	a.n = (uint32_t)c->n[axis];
	a.row_len = c->row_len;
	a.pitch = c->pitch;
	a.rows = c->rows;
	a.err = static_cast<uint32_t*>(c->err.ptr);
	a.ticket = static_cast<uint32_t*>(c->tickets.ptr) + axis;
	a.blo_off = c->coef_blo_off[axis];
	return a;
}

template <typename T, int MC>
int dispatch_sweep_x(Context* c, const SweepArgs& a, const Plan& p, bool sub)
{
	const double bytes = 2.0 * (double)(c->V * c->S) * (double)sizeof(T);
	if (sub)
		switch (c->S)
		{
		case 3: return launch_persistent(c, sweep_x_sub_kernel<T, 3, MC>, a, p, K_SWEEP_X, bytes);
		case 4: return launch_persistent(c, sweep_x_sub_kernel<T, 4, MC>, a, p, K_SWEEP_X, bytes);
		case 5: return launch_persistent(c, sweep_x_sub_kernel<T, 5, MC>, a, p, K_SWEEP_X, bytes);
		case 6: return launch_persistent(c, sweep_x_sub_kernel<T, 6, MC>, a, p, K_SWEEP_X, bytes);
		case 7: return launch_persistent(c, sweep_x_sub_kernel<T, 7, MC>, a, p, K_SWEEP_X, bytes);
		case 8: return launch_persistent(c, sweep_x_sub_kernel<T, 8, MC>, a, p, K_SWEEP_X, bytes);
		default: return launch_persistent(c, sweep_x_sub_kernel<T, 0, MC>, a, p, K_SWEEP_X, bytes);
		}
	switch (c->S)
	{
	case 1: return launch_persistent(c, sweep_x_kernel<T, 1, MC>, a, p, K_SWEEP_X, bytes);
	case 2: return launch_persistent(c, sweep_x_kernel<T, 2, MC>, a, p, K_SWEEP_X, bytes);
	case 3: return launch_persistent(c, sweep_x_kernel<T, 3, MC>, a, p, K_SWEEP_X, bytes);
	case 4: return launch_persistent(c, sweep_x_kernel<T, 4, MC>, a, p, K_SWEEP_X, bytes);
	case 5: return launch_persistent(c, sweep_x_kernel<T, 5, MC>, a, p, K_SWEEP_X, bytes);
	case 6: return launch_persistent(c, sweep_x_kernel<T, 6, MC>, a, p, K_SWEEP_X, bytes);
	case 7: return launch_persistent(c, sweep_x_kernel<T, 7, MC>, a, p, K_SWEEP_X, bytes);
	case 8: return launch_persistent(c, sweep_x_kernel<T, 8, MC>, a, p, K_SWEEP_X, bytes);
	default: return launch_persistent(c, sweep_x_kernel<T, 0, MC>, a, p, K_SWEEP_X, bytes);
	}
}

template <typename T>
int run_sweep_x(Context* c, bool mass_check)
{
	SweepArgs a = base_args(c, 0);
	const bool sub = x_substrate_mapping(c->S);
	a.smem_pitch = sub ? sweep_x_sub_pitch(c->row_len, c->S, sizeof(T)) : sweep_x_smem_pitch(c->row_len, c->S, sizeof(T));
	a.comp_off = c->coef_comp_off[0];
	a.head = c->coef_head[0];
	const Plan p = plan<T>(c, 0);
	if (p.smem > kMaxSmemBytes)
		return fail(PCG_ERR_UNSUPPORTED, "x rows too long for the shared-memory x sweep");
	a.rows_per_tile = (uint32_t)p.rows_per_tile;
	a.tiles = (c->rows + p.rows_per_tile - 1) / p.rows_per_tile;
	if (!mass_check)
		return dispatch_sweep_x<T, 0>(c, a, p, sub);
	a.mc_tot = static_cast<double*>(c->mc_tot.ptr);
	a.mc_x_out = c->dims == 1 ? 1u : 0u;
	// on a 1-D mesh x is also the last sweep: it sums its outputs as well
	return c->dims == 1 ? dispatch_sweep_x<T, kMcIn | kMcOut>(c, a, p, sub) : dispatch_sweep_x<T, kMcIn>(c, a, p, sub);
}

// The fused x + y launch (sweep_xy_kernel): slabs of about c->xy_slab_bytes of
// planes, y lagging x by at least c->xy_lag slabs and by at least twice the
// tiles the resident CTAs hold.  The segment table is rebuilt when the slab plan
// changes.
template <typename T>
int run_sweep_xy(Context* c, bool mass_check)
{
	SweepArgs ax = base_args(c, 0);
	ax.smem_pitch = sweep_x_sub_pitch(c->row_len, c->S, sizeof(T));
	ax.comp_off = c->coef_comp_off[0];
	ax.head = c->coef_head[0];
	const Plan px = plan<T>(c, 0);
	ax.rows_per_tile = (uint32_t)px.rows_per_tile;
	if (mass_check)
		ax.mc_tot = static_cast<double*>(c->mc_tot.ptr);
	SweepArgs ay = base_args(c, 1);
	ay.xblocks = (c->row_len + kLanes - 1) / kLanes;
	ay.box_rows = c->tmap_box_rows[1];
	ay.boxes = c->tmap_boxes[1];
	ay.comp_off = c->coef_comp_off[1];
	ay.head = c->coef_head[1];
	const Plan py = plan<T>(c, 1);
	const uint64_t R = px.rows_per_tile, ny = c->n[1], nz = c->n[2];
	const uint64_t plane_bytes = ny * c->pitch * sizeof(T);
	const uint64_t P = std::max<uint64_t>(1, std::min<uint64_t>(nz, c->xy_slab_bytes / plane_bytes));
	const uint64_t nslab = (nz + P - 1) / P;
	// the persistent grid (every CTA holds one tile at a time)
	const uint64_t smem = 128 + std::max(px.smem - 16, py.smem - 128);
	if (smem > kMaxSmemBytes)
		return fail(PCG_ERR_UNSUPPORTED, "fused x/y tiles too large for shared memory");
	auto kernel = [&]() -> void (*)(SweepArgs, SweepArgs, const CUtensorMap, XYArgs) {
		const bool mc = mass_check;
		switch (c->S)
		{
		case 3: return mc ? sweep_xy_kernel<T, 3, kMcIn> : sweep_xy_kernel<T, 3, 0>;
		case 4: return mc ? sweep_xy_kernel<T, 4, kMcIn> : sweep_xy_kernel<T, 4, 0>;
		case 5: return mc ? sweep_xy_kernel<T, 5, kMcIn> : sweep_xy_kernel<T, 5, 0>;
		case 6: return mc ? sweep_xy_kernel<T, 6, kMcIn> : sweep_xy_kernel<T, 6, 0>;
		case 7: return mc ? sweep_xy_kernel<T, 7, kMcIn> : sweep_xy_kernel<T, 7, 0>;
		case 8: return mc ? sweep_xy_kernel<T, 8, kMcIn> : sweep_xy_kernel<T, 8, 0>;
		default: return mc ? sweep_xy_kernel<T, 0, kMcIn> : sweep_xy_kernel<T, 0, 0>;
		}
	}();
	PCG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	int per_sm = 0;
	PCG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kLanes, smem));
	if (per_sm < 1)
		return fail(PCG_ERR_UNSUPPORTED, "fused x/y tile does not fit in shared memory");
	const uint64_t resident = (uint64_t)per_sm * (uint64_t)c->sm_count;
	// the lag must exceed the tiles in flight (about one per resident CTA), else y
	// tiles are handed out while their slab's x tiles are still being solved
	const uint64_t slab_tiles = (P * ny + R - 1) / R + P * ay.xblocks;
	const uint64_t L =
		std::max<uint64_t>(std::max<uint32_t>(1, c->xy_lag), (2 * resident + slab_tiles - 1) / slab_tiles);
	const uint64_t key = P | (L << 20) | (R << 40);
	if (c->xy_key != key || !c->xy_segs.ptr)
	{
		std::vector<uint4> segs;
		uint64_t first = 0;
		std::vector<uint32_t> tx(nslab);
		for (uint64_t k = 0; k < nslab + L; k++)
		{
			if (k < nslab)
			{
				const uint64_t rows_k = (std::min((k + 1) * P, nz) - k * P) * ny;
				tx[k] = (uint32_t)((rows_k + R - 1) / R);
				segs.push_back({ (uint32_t)first, (uint32_t)k, tx[k], 0u });
				first += tx[k];
			}
			if (k >= L)
			{
				const uint64_t j = k - L;
				const uint64_t ty = (std::min((j + 1) * P, nz) - j * P) * ay.xblocks;
				segs.push_back({ (uint32_t)first, (uint32_t)j | kYSeg, (uint32_t)ty, tx[j] });
				first += ty;
			}
		}
		if (first >= 0xffffffffull)
			return fail(PCG_ERR_UNSUPPORTED, "too many tiles for the fused x/y sweep");
		int rc;
		if ((rc = dalloc(c, c->xy_segs, segs.size() * sizeof(uint4))) ||
			(rc = dalloc(c, c->xy_done, nslab * sizeof(uint32_t))))
			return rc;
		PCG_CUDA_TRY(cudaMemcpyAsync(c->xy_segs.ptr, segs.data(), segs.size() * sizeof(uint4), cudaMemcpyHostToDevice,
									 c->stream));
		PCG_CUDA_TRY(stream_wait(c)); // the host table dies at scope exit
		c->xy_key = key;
		c->xy_nseg = (uint32_t)segs.size();
		c->xy_total = (uint32_t)first;
		c->xy_nslab = (uint32_t)nslab;
	}
	XYArgs f {};
	f.segs = static_cast<const uint4*>(c->xy_segs.ptr);
	f.nseg = c->xy_nseg;
	f.total = c->xy_total;
	f.planes = (uint32_t)P;
	f.done = static_cast<uint32_t*>(c->xy_done.ptr);
	f.ticket = static_cast<uint32_t*>(c->tickets.ptr) + 3;
	f.ny = ny;
	f.nz = nz;
	const uint64_t grid = std::min<uint64_t>(resident, c->xy_total);
	PCG_CUDA_TRY(cudaMemsetAsync(f.ticket, 0, sizeof(uint32_t), c->stream));
	PCG_CUDA_TRY(cudaMemsetAsync(f.done, 0, c->xy_nslab * sizeof(uint32_t), c->stream));
	// minimal traffic of the two sweeps: the field read once and written once
	const double bytes = 2.0 * (double)(c->V * c->S) * (double)sizeof(T);
	cudaEvent_t ev;
	launch_begin(c, K_SWEEP_XY, bytes, &ev);
	kernel<<<(unsigned)grid, kLanes, smem, c->stream>>>(ax, ay, c->tmap[1], f);
	launch_end(c, K_SWEEP_XY, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

template <typename T>
int run_sweep_yz(Context* c, int axis, bool fuse_faces, bool mass_check)
{
	SweepArgs a = base_args(c, axis);
	if (mass_check)
		a.mc_tot = static_cast<double*>(c->mc_tot.ptr);
	if (fuse_faces)
	{
		const FaceArgs f = make_face_args(c);
		a.face_values = f.values;
		a.face_conds = f.conds;
		a.face_mask = f.face_mask;
		a.nx = c->n[0], a.ny = c->n[1], a.nz = c->n[2];
	}
	if (axis == 1)
	{
		a.line_stride = c->pitch;
		a.outer_stride = c->n[1] * c->pitch;
		a.tiles = c->n[2];
	}
	else
	{
		a.line_stride = c->n[1] * c->pitch;
		a.outer_stride = c->pitch;
		a.tiles = c->n[1];
	}
	a.xblocks = (c->row_len + kLanes - 1) / kLanes;
	a.tiles *= a.xblocks;
	a.box_rows = c->tmap_box_rows[axis];
	a.boxes = c->tmap_boxes[axis];
	a.comp_off = c->coef_comp_off[axis];
	a.head = c->coef_head[axis];
	const Plan p = plan<T>(c, axis);
	if (p.smem > kMaxSmemBytes)
		return fail(PCG_ERR_UNSUPPORTED, "lines too long for the shared-memory y/z sweep");
	if (a.box_rows == 0)
		return fail(PCG_ERR_INVALID, "tensor maps of the field were not prepared");
	const int kid = axis == 1 ? K_SWEEP_Y : K_SWEEP_Z;
	const double bytes = 2.0 * (double)(c->V * c->S) * (double)sizeof(T);
	auto kernel = mass_check ? (axis == 1 ? sweep_yz_kernel<T, 1, kMcOut> : sweep_yz_kernel<T, 2, kMcOut>)
							 : (axis == 1 ? sweep_yz_kernel<T, 1, 0> : sweep_yz_kernel<T, 2, 0>);
	PCG_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p.smem));
	int per_sm = 0;
	PCG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, p.threads, p.smem));
	if (per_sm < 1)
		return fail(PCG_ERR_UNSUPPORTED, "sweep tile does not fit in shared memory");
	uint64_t grid = (uint64_t)per_sm * (uint64_t)c->sm_count;
	if (grid > a.tiles)
		grid = a.tiles;
	PCG_CUDA_TRY(cudaMemsetAsync(a.ticket, 0, sizeof(uint32_t), c->stream));
	cudaEvent_t ev;
	launch_begin(c, kid, bytes, &ev);
	kernel<<<(unsigned)grid, p.threads, p.smem, c->stream>>>(a, c->tmap[axis]);
	launch_end(c, kid, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
								   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
								   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
	static EncodeTiledFn fn = nullptr;
	if (!fn)
	{
		void* p = nullptr;
		cudaDriverEntryPointQueryResult q {};
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
				cudaSuccess &&
			q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<EncodeTiledFn>(p);
	}
	return fn;
}

} // namespace

// -------------------------------------------------------------------- host side

// Box geometry of a y/z tile: the fewest TMA boxes of at most 256 points (the box
// limit) that cover a line, each a multiple of the solver block, with the least
// padding.
void box_geometry(uint64_t n, uint32_t& box_rows, uint32_t& boxes)
{
	const uint64_t nc = (n + 255) / 256;
	boxes = (uint32_t)nc;
	box_rows = (uint32_t)round_up((n + nc - 1) / nc, 8);
}

uint64_t coef_table_len(uint64_t n, uint64_t S, size_t wsize)
{
	const int vn = (int)(16 / wsize);
	return round_up(n * S, (uint64_t)group_elems((int)S, vn));
}

uint64_t coef_row_pitch(uint64_t n) { return round_up(n, kBlock); }

uint64_t x_threads_per_row(uint64_t S, size_t wsize)
{
	return (S <= 8 && (S * wsize) % 16 == 0) ? S * wsize / 16 : 1;
}

bool x_substrate_mapping(uint64_t S) { return S >= 3 && S <= kLanes; }

// Shared-memory row pitch (elements) of the substrate-per-thread x mapping: whole
// 16-byte chunks, and rows S elements (rounded up to a chunk) apart modulo the 32
// banks, so that lane (r, s) of a warp reads bank r*S + s (mod 32) for FP32.
uint64_t sweep_x_sub_pitch(uint64_t row_len, uint64_t S, size_t wsize)
{
	const uint64_t vn = 16 / wsize;
	const uint64_t mod = 128 / wsize; // elements spanning the 32 banks
	const uint64_t want = round_up(S, vn) % mod;
	uint64_t p = round_up(row_len, vn);
	while (p % mod != want)
		p += vn;
	return p;
}

uint64_t sweep_x_smem_pitch(uint64_t row_len, uint64_t S, size_t wsize)
{
	const uint64_t vn = 16 / wsize;
	const uint64_t ge = (uint64_t)group_elems((int)S, (int)vn);
	const uint64_t tpr = x_threads_per_row(S, wsize);
	uint64_t chunks = round_up(row_len, ge) / vn;
	// rows tpr (mod 8) chunks apart: the 8 lanes of a quarter-warp (8/tpr rows x tpr
	// chunk slots) read 8 distinct 16-byte bank groups
	const uint64_t want = tpr % 8;
	chunks += (want + 8 - chunks % 8) % 8;
	return chunks * vn;
}

int encode_field_map(const Context* c, int axis, uint32_t box_rows, CUtensorMap* out, uint32_t box_cols)
{
	EncodeTiledFn enc = encode_fn();
	if (!enc)
		return fail(PCG_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
	const cuuint64_t dims[3] = { c->row_len, c->n[1], c->n[2] };
	const cuuint64_t strides[2] = { c->pitch * c->wsize, c->n[1] * c->pitch * c->wsize };
	const cuuint32_t estr[3] = { 1, 1, 1 };
	const CUtensorMapDataType dt = c->wsize == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
	const cuuint32_t box[3] = { box_cols, axis == 1 ? box_rows : 1u, axis == 2 ? box_rows : 1u };
	CUresult r = enc(out, dt, 3, c->field.ptr, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
					 CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
	if (r != CUDA_SUCCESS)
		return fail(PCG_ERR_CUDA, "cuTensorMapEncodeTiled failed with code " + std::to_string((int)r));
	return PCG_OK;
}

// Encodes the TMA tensor maps of the y and z sweeps for the current field buffer.
int prepare_sweep_maps(Context* c)
{
	for (int axis = 1; axis < c->dims; axis++)
	{
		uint32_t box_rows, boxes;
		box_geometry(c->n[axis], box_rows, boxes);
		const int rc = encode_field_map(c, axis, box_rows, &c->tmap[axis]);
		if (rc)
			return rc;
		c->tmap_box_rows[axis] = box_rows;
		c->tmap_boxes[axis] = boxes;
	}
	return PCG_OK;
}

uint64_t sweep_smem_bytes(const Context* c, int axis)
{
	return c->wsize == 4 ? plan<float>(c, axis).smem : plan<double>(c, axis).smem;
}

int launch_sweep_x(Context* c, bool mass_check)
{
	return c->wsize == 4 ? run_sweep_x<float>(c, mass_check) : run_sweep_x<double>(c, mass_check);
}

bool xy_fusable(const Context* c) { return c->fuse_xy && c->dims == 3 && x_substrate_mapping(c->S) && c->n[2] > 1; }

int launch_sweep_xy(Context* c, bool mass_check)
{
	return c->wsize == 4 ? run_sweep_xy<float>(c, mass_check) : run_sweep_xy<double>(c, mass_check);
}

int launch_sweep_yz(Context* c, int axis, bool fuse_faces, bool mass_check)
{
	return c->wsize == 4 ? run_sweep_yz<float>(c, axis, fuse_faces, mass_check)
						 : run_sweep_yz<double>(c, axis, fuse_faces, mass_check);
}

bool faces_fusable(const Context* c) { return c->dims >= 2; }

} // namespace pcg
