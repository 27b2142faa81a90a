// batch.cu -- many independent BioFVM domains stepped together on one GPU.
//
// The reference steps one microenvironment per solver call
// (openmp_solver/src/openmp_solver.cpp:23-40): diffusion x/y/z, Dirichlet, bulk,
// cells.  For many small domains of uneven size, one launch per phase per domain
// leaves the GPU idle between tiny grids and is bound by launch latency.  Here a
// batch keeps a device table of domain descriptors (each pointing at its
// context's own field, coefficient tables, Dirichlet sets, bulk tables and
// agents) and runs every phase as ONE launch over all domains:
//
//  * sweeps: one persistent launch per axis.  The tiles of all domains form one
//    list (domains ordered by decreasing tile cost); CTAs take tiles from an
//    atomic counter, find the tile's domain by binary search over the list's
//    prefix sums, and solve it with the domain's own line mapping and tile shape.
//    y/z tiles move through the domain's TMA tensor map (kept in global memory),
//    one mbarrier per chunk, so solving starts when the first chunk lands.
//  * Dirichlet faces/interior, bulk and the cell phases: one launch each over the
//    concatenated items of all domains (face voxels, interior nodes, rows, agents).
//  * the whole step is captured once in a CUDA graph and replayed.
//
// Per-domain arithmetic and phase order are exactly those of the single-domain
// kernels (the per-item device code is shared: sweep_solvers.cuh,
// field_device.cuh, cells_device.cuh), so a batched domain matches pcg_solve on
// the same context up to the order of floating-point atomic sums in the ballot.
//
// Autotuner: per sweep axis and size bucket (line length rounded up to 16, and
// for x the substrate count) candidate mappings are timed on the batch's own
// domains (fields saved and restored) and the fastest is kept for the process.
//   x:   row-per-thread (one thread carries all S recurrences of a row, walking it
//        as 16-byte chunks) or substrate-per-thread (S lanes share a row, one
//        recurrence each), times rows per tile;
//   y/z: points per TMA chunk (how early a line's solve can start vs. how many
//        copies a tile takes).
#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include "cells_device.cuh"
#include "field_device.cuh"
#include "pcg_internal.cuh"
#include "sweep_solvers.cuh"

namespace pcg {

namespace {

using namespace solvers;
using namespace cellsdev;

enum : uint32_t
{
	kMapRow = 0,       // x: a thread owns a row (all substrates)
	kMapSubstrate = 1, // x: a thread owns one substrate of a row
	kMapColumn = 0,    // y/z: a lane owns one (x,s) column
};

constexpr uint32_t kMaxChunks = 64;        // y/z boxes per line (TMA operations per tile)
constexpr uint64_t kClearChunk = 4096;     // voxels of the ballot counts cleared per warp item
constexpr uint64_t kXSmemDefault = 32768;  // default shared-memory budget of an x tile
constexpr double kTuneShare = 0.01;        // buckets below this share of an axis keep the defaults
constexpr uint64_t kGroupBytes = 16 * 1024; // y/z: tiles of a domain taken together up to this many bytes,
											 // or up to the batch's largest tile when that is larger
constexpr uint32_t kMaxGroup = 8;

struct BatchDomain
{
	void* field;
	uint64_t pitch, row_len, rows, V;
	uint32_t S, dims;
	uint32_t n[3];
	uint32_t x_rows; // rows per x tile
	uint32_t x_mode; // kMapRow or kMapSubstrate
	uint64_t x_smem_pitch;
	uint32_t box_rows[3], boxes[3];
	uint64_t yz_xblocks;       // y/z: tiles across a row (32 elements each)
	uint32_t yz_group[3];      // y/z: consecutive tiles per work unit (short lines share a CTA's buffer)
	const void* coef[3];
	uint64_t coef_len[3];
	uint64_t coef_comp_off[3]; // compressed tables (elements into coef)
	uint64_t coef_blo_off[3];  // FP32: full tables of the multipliers' lo parts (elements into coef)
	uint32_t coef_head[3];     // head points of the compressed tables
	FaceArgs faces;
	const uint64_t* dir_offsets;
	const void* dir_values;
	const uint8_t* dir_conds;
	uint64_t K;
	int bulk_mode;
	const void* bulk[3];
	double dt;
	CellArgs cells;
	// per-step mass check of this domain (null when off): FP64 totals [before S |
	// after S] added by the sweeps, and [before | after | worst | factor] x S
	double* mc_tot;
	double* mc_out;
};

// Entry k of a list covers units [base[k], base[k+1]) of domain dom[k].
struct WorkList
{
	const uint64_t* base;
	const uint32_t* dom;
	const uint32_t* hint; // hint[j]: the entry holding unit j << shift
	uint32_t count;
	uint32_t shift;
	uint64_t total;
};

struct BatchArgs
{
	const BatchDomain* doms;
	const CUtensorMap* tmaps; // [domain][2]: y, z
	WorkList list;
	uint32_t* counter;        // tile counter of this launch (zeroed at the start of every step)
	uint32_t* err;            // [0] DEV_ERR_* bits, [1] lowest failing domain
	const uint8_t* recompute; // per domain: rebuild the ballot this step
	uint32_t* steps_left;     // per domain: steps still to run in this call (0: the domain sits out)
};

// The entry holding unit u < total: from the hint of u's block, forward over the
// entries that start inside the block (usually none or one), instead of a binary
// search's chain of dependent loads.
__device__ __forceinline__ uint32_t find_entry(const WorkList& l, uint64_t u)
{
	uint32_t k = __ldg(l.hint + (u >> l.shift));
	while (k + 1 < l.count && __ldg(l.base + k + 1) <= u)
		k++;
	return k;
}

// find_entry for the 32 lanes of a warp holding ascending units (all lanes must
// call it): lane 0 searches once and the others step forward from its entry,
// usually not at all, since consecutive units rarely cross a domain.  Units past
// the list's end map to its last entry.
__device__ __forceinline__ uint32_t warp_entry(const WorkList& l, uint64_t u)
{
	const uint64_t uc = u < l.total ? u : l.total - 1;
	const uint64_t u0 = __shfl_sync(0xffffffffu, uc, 0);
	uint32_t k = 0;
	if ((threadIdx.x & 31) == 0)
		k = find_entry(l, u0);
	k = __shfl_sync(0xffffffffu, k, 0);
	while (k + 1 < l.count && __ldg(l.base + k + 1) <= uc)
		k++;
	return k;
}

__device__ __forceinline__ void report(const BatchArgs& b, uint32_t bits, uint32_t d)
{
	atomicOr(b.err, bits);
	atomicMin(b.err + 1, d);
}

__device__ __forceinline__ void fence_tensormap_acquire(const void* map)
{
	asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(map) : "memory");
}

// ------------------------------------------------------------------ sweeps

// Row-per-thread x solver of the batch: one thread carries the ST recurrences of
// a row, walking it in groups of lcm(ST, VN) elements (whole 16-byte chunks, so
// each element's substrate is a compile-time index).  A group's chunks and
// coefficients are loaded together; there is no cross-group prefetch, which keeps
// every substrate variant light enough to share one kernel (batched tiles are
// small, so many CTAs per SM hide the latency instead).
// MC adds substrate s's inputs / outputs to acc_in[s] / acc_out[s].
template <typename T, int ST, int MC = 0>
__device__ __forceinline__ void solve_row_lite(T* row, const T* __restrict__ cB, const T* __restrict__ cE,
											   const T* __restrict__ cC, const T* __restrict__ cBl, uint32_t n,
											   MassAcc<T>* acc_in = nullptr, MassAcc<T>* acc_out = nullptr)
{
	constexpr bool kLo = sizeof(T) == 4;
	using V = typename Vec16<T>::type;
	constexpr int VN = Vec16<T>::N;
	constexpr int GE = group_elems(ST, VN);
	constexpr int U = GE / VN;
	const uint32_t total = n * ST;
	const uint32_t groups = (total + GE - 1) / GE;
	V* __restrict__ vrow = reinterpret_cast<V*>(row);
	const V* vE = reinterpret_cast<const V*>(cE);
	const V* vB = reinterpret_cast<const V*>(cB);
	T d[ST], c[ST];
#pragma unroll
	for (int s = 0; s < ST; s++)
	{
		d[s] = T(0);
		c[s] = __ldg(cC + s);
	}
	for (uint32_t g = 0; g < groups; g++)
	{
		V x[U], e[U];
#pragma unroll
		for (int q = 0; q < U; q++)
		{
			x[q] = vrow[g * U + q];
			e[q] = __ldg(vE + g * U + q);
		}
#pragma unroll
		for (int q = 0; q < U; q++)
#pragma unroll
			for (int u = 0; u < VN; u++)
			{
				const int s = (q * VN + u) % ST;
				if (g * GE + q * VN + u < total)
				{
					if constexpr ((MC & kMcIn) != 0)
						acc_in[s].add(vget<V, T>(x[q], u));
					d[s] = dev::fmadd(vget<V, T>(e[q], u), d[s], vget<V, T>(x[q], u));
					vset<V, T>(x[q], u, d[s]);
				}
			}
#pragma unroll
		for (int q = 0; q < U; q++)
			vrow[g * U + q] = x[q];
	}
#pragma unroll
	for (int s = 0; s < ST; s++)
		d[s] = T(0);
	for (int g = (int)groups - 1; g >= 0; g--)
	{
		V x[U], bb[U], bl[U];
#pragma unroll
		for (int q = 0; q < U; q++)
		{
			x[q] = vrow[g * U + q];
			bb[q] = __ldg(vB + g * U + q);
			if constexpr (kLo)
				bl[q] = __ldg(reinterpret_cast<const V*>(cBl) + g * U + q);
		}
#pragma unroll
		for (int q = U - 1; q >= 0; q--)
#pragma unroll
			for (int u = VN - 1; u >= 0; u--)
			{
				const int s = (q * VN + u) % ST;
				if ((uint32_t)g * GE + q * VN + u < total)
				{
					d[s] = bwd_step(c[s], d[s], vget<V, T>(x[q], u), vget<V, T>(bb[q], u),
									kLo ? vget<V, T>(bl[q], u) : T(0));
					vset<V, T>(x[q], u, d[s]);
					if constexpr ((MC & kMcOut) != 0)
						acc_out[s].add(d[s]);
				}
			}
#pragma unroll
		for (int q = 0; q < U; q++)
			vrow[g * U + q] = x[q];
	}
}

// One row per thread; `active` threads hold a row.  With MC every thread of the
// warp calls it (the mass totals are summed across the warp): the rows' input
// totals go to mc_in[s] and, when mc_out is given (x is the domain's last
// sweep), their output totals to mc_out[s].
template <typename T, int ST, int MC>
__device__ __forceinline__ void solve_x_row_st(T* row, const T* cB, const T* cE, const T* cC, const T* cBl, uint32_t n,
											   bool active, double* mc_in, double* mc_out)
{
	MassAcc<T> ai[ST], ao[ST];
#pragma unroll
	for (int s = 0; s < ST; s++)
	{
		ai[s].zero();
		ao[s].zero();
	}
	if (active)
		solve_row_lite<T, ST, MC>(row, cB, cE, cC, cBl, n, ai, ao);
	if constexpr (MC != 0)
	{
#pragma unroll
		for (int s = 0; s < ST; s++)
		{
			if (mc_in)
				flush_classes(ai[s].value(), 1, kLanes, mc_in + s);
			if (mc_out)
				flush_classes(ao[s].value(), 1, kLanes, mc_out + s);
		}
	}
}

template <typename T, int MC>
__device__ __forceinline__ void solve_x_row(T* row, const T* cB, const T* cE, const T* cC, const T* cBl, uint32_t n,
											uint32_t S, bool active, double* mc_in, double* mc_out)
{
	switch (S)
	{
	case 1: solve_x_row_st<T, 1, MC>(row, cB, cE, cC, cBl, n, active, mc_in, mc_out); break;
	case 2: solve_x_row_st<T, 2, MC>(row, cB, cE, cC, cBl, n, active, mc_in, mc_out); break;
	case 3: solve_x_row_st<T, 3, MC>(row, cB, cE, cC, cBl, n, active, mc_in, mc_out); break;
	case 4: solve_x_row_st<T, 4, MC>(row, cB, cE, cC, cBl, n, active, mc_in, mc_out); break;
	case 5: solve_x_row_st<T, 5, MC>(row, cB, cE, cC, cBl, n, active, mc_in, mc_out); break;
	case 6: solve_x_row_st<T, 6, MC>(row, cB, cE, cC, cBl, n, active, mc_in, mc_out); break;
	case 7: solve_x_row_st<T, 7, MC>(row, cB, cE, cC, cBl, n, active, mc_in, mc_out); break;
	case 8: solve_x_row_st<T, 8, MC>(row, cB, cE, cC, cBl, n, active, mc_in, mc_out); break;
	default:
		if (active)
			solve_row_generic<T, MC>(row, cB, cE, cC, cBl, n, S, mc_in, mc_out);
		break;
	}
}

// x: a tile is x_rows whole rows of one domain, bulk-copied into shared memory.
// MC (mass check in this batch): for domains with the check on, the tile's input
// totals (and output totals when x is the domain's last sweep) go to its mc_tot.
template <typename T, int MC>
__global__ void __launch_bounds__(kLanes) batch_sweep_x_kernel(BatchArgs b)
{
	extern __shared__ __align__(128) unsigned char smem[];
	uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
	T* tile = reinterpret_cast<T*>(smem + 16);
	const uint32_t tid = threadIdx.x;
	if (tid == 0)
	{
		dev::mbar_init(bar, 1);
		dev::fence_mbar_init();
	}
	__syncthreads();
	uint32_t phase = 0;
	uint32_t next = 0;
	if (tid == 0)
		next = atomicAdd(b.counter, 1u);
	// A unit's work-list entry and domain are resolved while the previous unit's
	// rows load, and a new domain's descriptor is prefetched into L1 then (the CTA
	// is one warp).
	auto resolve = [&](uint64_t u, uint32_t& k, uint32_t& di) {
		k = di = 0;
		if (u < b.list.total)
		{
			k = find_entry(b.list, u);
			di = __ldg(b.list.dom + k);
		}
	};
	uint64_t t = __shfl_sync(0xffffffffu, next, 0);
	uint32_t k, di;
	resolve(t, k, di);
	for (;;)
	{
		if (t >= b.list.total)
			break;
		if (tid == 0)
			next = atomicAdd(b.counter, 1u); // the following tile's ticket, in flight meanwhile
		if (b.steps_left[di] == 0)
		{
			t = __shfl_sync(0xffffffffu, next, 0);
			resolve(t, k, di);
			continue;
		}
		const BatchDomain& D = b.doms[di];
		const uint32_t R = D.x_rows, S = D.S, n = D.n[0];
		const uint64_t r0 = (t - __ldg(b.list.base + k)) * R;
		const uint32_t nrows = (uint32_t)min((uint64_t)R, D.rows - r0);
		const uint32_t row_bytes = (uint32_t)round_up(D.row_len * sizeof(T), 16);
		const uint64_t spitch = D.x_smem_pitch;
		T* g = static_cast<T*>(D.field) + r0 * D.pitch;
		if (tid == 0)
			dev::mbar_arrive_expect_tx(bar, nrows * row_bytes);
		__syncthreads();
		if (tid < nrows)
			dev::bulk_g2s(tile + tid * spitch, g + tid * D.pitch, row_bytes, bar);
		const uint64_t tn = __shfl_sync(0xffffffffu, next, 0);
		uint32_t kn, dn;
		resolve(tn, kn, dn);
		if (dn != di && tid * 128 < sizeof(BatchDomain))
			asm volatile("prefetch.global.L1 [%0];" ::"l"(reinterpret_cast<const char*>(b.doms + dn) + tid * 128));
		const T* cB = static_cast<const T*>(D.coef[0]);
		const T* cE = cB + D.coef_len[0];
		const T* cC = cE + D.coef_len[0];
		const T* cBl = sizeof(T) == 4 ? cB + D.coef_blo_off[0] : nullptr;
		const uint32_t rl = tid / S, s = tid % S;
		LineCoef<T> L {};
		if (D.x_mode != kMapRow) // coefficient loads overlap the tile's arrival
			L = line_coef<T>(static_cast<const T*>(D.coef[0]) + D.coef_comp_off[0], S, D.coef_head[0], n, s);
		const bool ok = __all_sync(0xffffffffu, dev::mbar_wait(bar, phase));
		if (!ok)
		{
			if (tid == 0)
				report(b, DEV_ERR_WAIT_TIMEOUT, di);
			return;
		}
		double* mc_in = MC != 0 ? D.mc_tot : nullptr;
		double* mc_out = MC != 0 && D.mc_tot && D.dims == 1 ? D.mc_tot + S : nullptr;
		if (D.x_mode == kMapRow)
			solve_x_row<T, MC>(tile + tid * spitch, cB, cE, cC, cBl, n, S, tid < nrows, mc_in, mc_out);
		else
		{
			MassAcc<T> ai, ao;
			ai.zero();
			ao.zero();
			if (rl < nrows)
				solve_line<T, 0, MC>(tile + rl * spitch + s, n, S, L, &ai, &ao);
			if constexpr (MC != 0)
			{
				// lanes rl * S + s share substrate s (S <= 32 on this mapping)
				if (mc_in)
					flush_classes(ai.value(), S, kLanes, mc_in + s % S);
				if (mc_out)
					flush_classes(ao.value(), S, kLanes, mc_out + s % S);
			}
		}
		dev::fence_proxy_async_smem();
		__syncthreads();
		if (tid < nrows)
			dev::bulk_s2g(g + tid * D.pitch, tile + tid * spitch, row_bytes);
		dev::bulk_commit();
		dev::bulk_wait_read();
		__syncthreads();
		phase ^= 1;
		t = tn;
		k = kn;
		di = dn;
	}
	dev::bulk_wait_all();
}

// y/z: a tile is 32 consecutive (x,s) columns at every point of one line
// set of one domain; its boxes arrive through the domain's tensor map on one
// mbarrier, the warp solves it in place, and the boxes are stored back before the
// next tile is requested (several single-warp CTAs per SM overlap these phases).
// MC (mass check in this batch): on the domain's last sweep, each tile's solved
// totals (before its faces are written) go to the domain's mc_tot.
template <typename T, int AXIS, int MC>
__global__ void __launch_bounds__(kLanes) batch_sweep_yz_kernel(BatchArgs b)
{
	extern __shared__ __align__(128) unsigned char smem[];
	uint64_t* full = reinterpret_cast<uint64_t*>(smem);
	T* base = reinterpret_cast<T*>(smem + 128);
	const uint32_t lane = threadIdx.x;
	if (lane == 0)
	{
		dev::mbar_init(full, 1);
		dev::fence_mbar_init();
	}
	__syncwarp();
	uint32_t phase = 0, prev = 0xffffffffu, bad = 0;
	bool ok = true;
	uint32_t next = 0;
	if (lane == 0)
		next = atomicAdd(b.counter, 1u);
	// A unit's work-list entry and domain are resolved while the previous unit's
	// tiles load, and a new domain's descriptor is prefetched into L1 then.
	auto resolve = [&](uint64_t u, uint32_t& k, uint32_t& di) {
		k = di = 0;
		if (u < b.list.total)
		{
			k = find_entry(b.list, u);
			di = __ldg(b.list.dom + k);
		}
	};
	uint64_t t = __shfl_sync(0xffffffffu, next, 0);
	uint32_t k, di;
	resolve(t, k, di);
	for (;; phase ^= 1)
	{
		if (t >= b.list.total)
			break;
		if (lane == 0)
			next = atomicAdd(b.counter, 1u); // the following tile's ticket, in flight meanwhile
		if (b.steps_left[di] == 0)
		{
			phase ^= 1; // no tile was loaded: keep the barrier's parity
			t = __shfl_sync(0xffffffffu, next, 0);
			resolve(t, k, di);
			continue;
		}
		const BatchDomain& D = b.doms[di];
		// a unit is `group` consecutive tiles of the domain (short lines: several
		// tiles share the buffer, so one ticket, lookup and wait serve them all)
		const uint32_t group = D.yz_group[AXIS];
		const uint64_t tiles = D.yz_xblocks * (AXIS == 1 ? D.n[2] : D.n[1]);
		const uint64_t lt0 = (t - __ldg(b.list.base + k)) * group;
		const uint32_t gcount = (uint32_t)min((uint64_t)group, tiles - lt0);
		const uint32_t R = D.box_rows[AXIS], nc = D.boxes[AXIS], n = D.n[AXIS], S = D.S;
		const uint32_t chunk_elems = R * kLanes, tile_elems = nc * chunk_elems;
		const CUtensorMap* map = b.tmaps + 2 * di + (AXIS - 1);
		// the unit's first tile (x block, outer index) by one 32-bit division per unit
		// (a domain has fewer than 2^32 tiles); the following tiles step from it, so
		// no tile's load, solve or store divides
		const uint32_t xblocks = (uint32_t)D.yz_xblocks;
		const uint32_t xb0 = (uint32_t)lt0 % xblocks, ob0 = (uint32_t)lt0 / xblocks;
		auto step_tile = [xblocks](uint32_t& xb, uint32_t& ob) {
			if (++xb == xblocks)
			{
				xb = 0;
				ob++;
			}
		};
		if (lane == 0)
		{
			if (di != prev)
				fence_tensormap_acquire(map);
			dev::mbar_arrive_expect_tx(full, gcount * tile_elems * (uint32_t)sizeof(T));
			uint32_t xb = xb0, ob = ob0;
			for (uint32_t j = 0; j < gcount; j++, step_tile(xb, ob))
			{
				const int x0 = (int)(xb * kLanes), o = (int)ob;
				for (uint32_t c = 0; c < nc; c++)
				{
					T* dst = base + j * tile_elems + c * chunk_elems;
					if (AXIS == 1)
						dev::tma_load_3d(dst, map, x0, (int)(c * R), o, full);
					else
						dev::tma_load_3d(dst, map, x0, o, (int)(c * R), full);
				}
			}
		}
		prev = di;
		const uint64_t tn = __shfl_sync(0xffffffffu, next, 0);
		uint32_t kn, dn;
		resolve(tn, kn, dn);
		if (dn != di && lane * 128 < sizeof(BatchDomain))
			asm volatile("prefetch.global.L1 [%0];" ::"l"(reinterpret_cast<const char*>(b.doms + dn) + lane * 128));
		const T* comp = static_cast<const T*>(D.coef[AXIS]) + D.coef_comp_off[AXIS];
		// the first tile's coefficient loads overlap the group's arrival
		uint32_t xb = xb0, ob = ob0;
		int x0 = (int)(xb * kLanes), o = (int)ob;
		LineCoef<T> L = line_coef<T>(comp, S, D.coef_head[AXIS], n,
									 (uint64_t)(x0 + lane) < D.row_len ? (uint32_t)((x0 + lane) % S) : 0);
		ok = __all_sync(0xffffffffu, dev::mbar_wait(full, phase));
		if (!ok)
		{
			bad = di;
			break;
		}
		for (uint32_t j = 0; j < gcount; j++)
		{
			if (j)
			{
				step_tile(xb, ob);
				x0 = (int)(xb * kLanes), o = (int)ob;
				L = line_coef<T>(comp, S, D.coef_head[AXIS], n,
								 (uint64_t)(x0 + lane) < D.row_len ? (uint32_t)((x0 + lane) % S) : 0);
			}
			MassAcc<T> acc;
			acc.zero();
			solve_line<T, kLanes, MC>(base + j * tile_elems + lane, n, 0, L, nullptr, &acc);
			if constexpr (MC != 0)
				if (D.mc_tot && D.dims == AXIS + 1)
					flush_classes(acc.value(), S < kLanes ? S : kLanes, kLanes,
								  D.mc_tot + S + ((uint32_t)x0 + lane) % S);
			// the last sweep of the domain writes its boundary faces (the batch's
			// Dirichlet launch then covers interior nodes and 1-D domains only)
			if (D.dims == AXIS + 1)
				fielddev::faces_on_column<T, AXIS>(D.faces, base + j * tile_elems + lane, n, kLanes,
												   (uint64_t)x0 + lane, (uint64_t)o);
		}
		dev::fence_proxy_async_smem();
		__syncwarp();
		if (lane == 0)
		{
			uint32_t xs_b = xb0, os_b = ob0;
			for (uint32_t j = 0; j < gcount; j++, step_tile(xs_b, os_b))
			{
				const int xs = (int)(xs_b * kLanes), os = (int)os_b;
				for (uint32_t c = 0; c < nc; c++)
				{
					T* src = base + j * tile_elems + c * chunk_elems;
					if (AXIS == 1)
						dev::tma_store_3d(map, xs, (int)(c * R), os, src);
					else
						dev::tma_store_3d(map, xs, os, (int)(c * R), src);
				}
			}
			dev::bulk_commit();
			dev::bulk_wait_read();
		}
		__syncwarp();
		t = tn;
		k = kn;
		di = dn;
	}
	if (!ok && lane == 0)
		report(b, DEV_ERR_WAIT_TIMEOUT, bad);
	if (lane == 0)
		dev::bulk_wait_all();
}

// ------------------------------------------------------------------ Dirichlet, bulk

// Grid-stride loops below step whole warps together (a warp's first unit decides),
// so that every lane takes part in warp_entry.
template <typename T>
__global__ void batch_faces_kernel(BatchArgs b)
{
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	const uint64_t w0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u);
	for (uint64_t wu = w0; wu < b.list.total; wu += stride)
	{
		const uint64_t u = wu + (threadIdx.x & 31);
		const uint32_t k = warp_entry(b.list, u);
		if (u < b.list.total && b.steps_left[__ldg(b.list.dom + k)])
			fielddev::face_item<T>(b.doms[__ldg(b.list.dom + k)].faces, u - __ldg(b.list.base + k));
	}
}

template <typename T>
__global__ void batch_interior_kernel(BatchArgs b)
{
	const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
	const uint64_t w0 = blockIdx.x * (uint64_t)blockDim.x + (threadIdx.x & ~31u);
	for (uint64_t wu = w0; wu < b.list.total; wu += stride)
	{
		const uint64_t u = wu + (threadIdx.x & 31);
		const uint32_t k = warp_entry(b.list, u);
		if (u >= b.list.total || !b.steps_left[__ldg(b.list.dom + k)])
			continue;
		const BatchDomain& D = b.doms[__ldg(b.list.dom + k)];
		const uint64_t i = u - __ldg(b.list.base + k);
		if (D.dir_conds[i])
			static_cast<T*>(D.field)[D.dir_offsets[i / D.S] + i % D.S] = static_cast<const T*>(D.dir_values)[i];
	}
}

// A warp per row of a domain with a bulk table.
template <typename T>
__global__ void batch_bulk_kernel(BatchArgs b)
{
	const int lane = threadIdx.x & 31;
	const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
	const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
	for (uint64_t u = warp; u < b.list.total; u += nwarps)
	{
		const uint32_t k = warp_entry(b.list, u);
		if (!b.steps_left[__ldg(b.list.dom + k)])
			continue;
		const BatchDomain& D = b.doms[__ldg(b.list.dom + k)];
		const uint64_t r = u - __ldg(b.list.base + k);
		const T* sp = static_cast<const T*>(D.bulk[0]);
		const T* up = static_cast<const T*>(D.bulk[1]);
		const T* tp = static_cast<const T*>(D.bulk[2]);
		if (D.bulk_mode == PCG_BULK_PER_VOXEL)
			fielddev::bulk_row<T, true>(static_cast<T*>(D.field), sp, up, tp, D.row_len, D.pitch, r, D.S, (T)D.dt,
										lane);
		else
			fielddev::bulk_row<T, false>(static_cast<T*>(D.field), sp, up, tp, D.row_len, D.pitch, r, D.S, (T)D.dt,
										 lane);
	}
}

// ------------------------------------------------------------------ cells

// Ballot counts of domains that rebuild their ballot this step: a warp clears
// kClearChunk voxels.
__global__ void batch_clear_counts_kernel(BatchArgs b)
{
	const int lane = threadIdx.x & 31;
	const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
	const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
	for (uint64_t u = warp; u < b.list.total; u += nwarps)
	{
		const uint32_t k = warp_entry(b.list, u);
		const uint32_t di = __ldg(b.list.dom + k);
		if (!b.recompute[di] || !b.steps_left[di])
			continue;
		const BatchDomain& D = b.doms[di];
		const uint64_t v0 = (u - __ldg(b.list.base + k)) * kClearChunk;
		const uint64_t v1 = min(v0 + kClearChunk, D.V);
		uint32_t* counts = D.cells.counts;
		for (uint64_t v = v0 + lane; v < v1; v += 32)
			counts[v] = 0;
	}
}

template <typename T>
__global__ void batch_cells_locate_kernel(BatchArgs b)
{
	const uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	const uint32_t k = warp_entry(b.list, u);
	if (u >= b.list.total)
		return;
	const uint32_t di = __ldg(b.list.dom + k);
	if (!b.recompute[di] || !b.steps_left[di])
		return;
	const CellArgs& a = b.doms[di].cells;
	const uint64_t i = u - __ldg(b.list.base + k);
	if (i == 0)
		a.flags[0] = a.flags[1] = 0;
	agent_locate<T>(a, i);
}

// Lanes of a warp may hold agents of two domains: the match key carries the domain.
__global__ void batch_cells_ballot_kernel(BatchArgs b)
{
	const uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	uint64_t key = ~0ull;
	uint32_t v = kNoAgent, di = 0;
	uint64_t i = 0;
	const uint32_t k = warp_entry(b.list, u);
	if (u < b.list.total)
	{
		di = __ldg(b.list.dom + k);
		if (b.recompute[di] && b.steps_left[di])
		{
			i = u - __ldg(b.list.base + k);
			v = b.doms[di].cells.vox[i];
			if (v != kNoAgent)
				key = ((uint64_t)di << 32) | v;
		}
	}
	const uint32_t group = __match_any_sync(0xffffffffu, key);
	if (key == ~0ull)
		return;
	if ((threadIdx.x & 31) == (uint32_t)(__ffs(group) - 1))
	{
		// consecutive lanes hold consecutive agents of a domain: the leader is the group minimum
		const CellArgs& a = b.doms[di].cells;
		atomicMin(a.owner + v, (uint32_t)i);
		atomicAdd(a.counts + v, (uint32_t)__popc(group));
	}
}

template <typename T>
__global__ void batch_cells_reduce_kernel(BatchArgs b)
{
	const uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	uint8_t role = kRoleNone;
	uint32_t di = 0;
	uint64_t i = 0;
	const uint32_t k = warp_entry(b.list, u);
	if (u < b.list.total)
	{
		di = __ldg(b.list.dom + k);
		if (b.recompute[di] && b.steps_left[di])
		{
			i = u - __ldg(b.list.base + k);
			role = agent_reduce<T>(b.doms[di].cells, i);
		}
	}
	const bool conflict = role == kRoleLoser;
	const uint32_t group = __match_any_sync(0xffffffffu, conflict ? di : 0xffffffffu);
	if (conflict && (threadIdx.x & 31) == (uint32_t)(__ffs(group) - 1))
		atomicOr(b.doms[di].cells.flags, 1u);
	list_shared(b.doms[di].cells, i, role == kRoleWinner || role == kRoleLoser, di);
}

// FP32: registers capped for 3 blocks of 256 per SM (a latency-bound gather:
// more loads in flight; the FP64 build would spill)
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) batch_cells_apply_kernel(BatchArgs b)
{
	const uint64_t u = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	const uint32_t k = warp_entry(b.list, u);
	if (u >= b.list.total || !b.steps_left[__ldg(b.list.dom + k)])
		return;
	agent_apply<T>(b.doms[__ldg(b.list.dom + k)].cells, u - __ldg(b.list.base + k));
}

template <typename T>
__global__ void batch_cells_internalize_kernel(BatchArgs b, const uint32_t* __restrict__ block0, uint32_t ndom)
{
	// Work is the domains' lists of agents in shared voxels, whose lengths are on
	// the device.  Domain d owns blocks [block0[d], block0[d+1]) (in proportion to
	// its agents, set when the batch is built) and splits its list among them.
	uint32_t lo = 0, hi = ndom; // the last d with block0[d] <= blockIdx.x
	while (hi - lo > 1)
	{
		const uint32_t mid = (lo + hi) / 2;
		if (__ldg(block0 + mid) <= blockIdx.x)
			lo = mid;
		else
			hi = mid;
	}
	const uint32_t d = lo;
	const uint32_t part = blockIdx.x - __ldg(block0 + d), parts = __ldg(block0 + d + 1) - __ldg(block0 + d);
	const CellArgs& a = b.doms[d].cells;
	if (!b.steps_left[d] || !a.internalized || !a.A || part >= parts)
		return;
	const uint32_t count = __ldg(a.flags + 1);
	for (uint64_t j = (uint64_t)part * blockDim.x + threadIdx.x; j < count; j += (uint64_t)parts * blockDim.x)
		agent_internalize<T>(a, __ldg(a.shared + j));
}

// After the sweeps of a step: for every domain with the mass check on that runs
// this step, the masses before and after its sweeps, the worst residual of
// after * factor = before, and its totals cleared for the next step.
__global__ void batch_mass_finish_kernel(const BatchDomain* doms, const uint32_t* steps_left, uint32_t count)
{
	for (uint32_t d = blockIdx.x; d < count; d += gridDim.x)
	{
		const BatchDomain& D = doms[d];
		if (!D.mc_tot || !steps_left[d])
			continue;
		const uint32_t S = D.S;
		for (uint32_t s = threadIdx.x; s < S; s += blockDim.x)
		{
			const double bf = D.mc_tot[s], af = D.mc_tot[S + s];
			D.mc_out[s] = bf;
			D.mc_out[S + s] = af;
			const double res = fabs(af * D.mc_out[3 * S + s] - bf) / fmax(fabs(bf), 1e-300);
			D.mc_out[2 * S + s] = fmax(D.mc_out[2 * S + s], res);
			D.mc_tot[s] = 0.0;
			D.mc_tot[S + s] = 0.0;
		}
	}
}

// Timing mode only: the algorithmic bytes of this step's internalize pass, which
// reads and rewrites the rows of the agents in shared voxels (their number is on
// the device): list entry, offset, density, own terms, internalized amount.
__global__ void batch_shared_bytes_kernel(const BatchDomain* doms, const uint32_t* steps_left, uint32_t count,
										  uint32_t wsize, double* out)
{
	double acc = 0.0;
	for (uint32_t d = threadIdx.x; d < count; d += blockDim.x)
	{
		const CellArgs& a = doms[d].cells;
		if (steps_left[d] && a.internalized && a.A)
			acc += (double)__ldg(a.flags + 1) * (8.0 + 4.0 * a.S * wsize + 16.0 * a.S);
	}
	for (int o = 16; o > 0; o >>= 1)
		acc += __shfl_xor_sync(0xffffffffu, acc, o);
	__shared__ double part[32];
	if ((threadIdx.x & 31) == 0)
		part[threadIdx.x >> 5] = acc;
	__syncthreads();
	if (threadIdx.x == 0)
	{
		double t = 0.0;
		for (uint32_t w = 0; w < blockDim.x / 32; w++)
			t += part[w];
		*out = t;
	}
}

// End of a step: one step fewer for every domain still running.
__global__ void batch_count_step_kernel(uint32_t* steps_left, uint32_t count)
{
	for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < count; d += gridDim.x * blockDim.x)
		if (steps_left[d])
			steps_left[d]--;
}

// ------------------------------------------------------------------ host side

enum ListId : int
{
	L_X = 0,
	L_Y,
	L_Z,
	L_FACES,
	L_INTERIOR,
	L_BULK,
	L_CLEAR,
	L_AGENTS,
	L_COUNT
};

struct AxisConfig
{
	uint32_t mode = kMapRow; // x only
	uint32_t rows = 0;       // x: rows per tile; y/z: points per chunk
	bool operator==(const AxisConfig& o) const { return mode == o.mode && rows == o.rows; }
};

struct TuneRecord
{
	int axis;
	double share; // of the axis' voxel-substrates
	uint64_t n_bucket, S, domains;
	AxisConfig best;
	double best_us;
	std::vector<std::pair<AxisConfig, double>> tried;
};

std::mutex g_tune_mu;
std::map<uint64_t, AxisConfig> g_tuned; // bucket key -> choice

uint64_t bucket_of(uint64_t n) { return round_up(n, 16); }

uint64_t bucket_key(int axis, size_t w, uint64_t S, uint64_t n)
{
	return (uint64_t)axis | (w == 8 ? 4ull : 0ull) | ((axis == 0 ? S : 0ull) << 3) | (bucket_of(n) << 16);
}

// Shared-memory pitch (elements) of a batched x row: whole vector groups, and an
// odd number of 16-byte chunks mod 8 (1), so the 8 lanes of a quarter-warp reading
// one chunk of 8 consecutive rows hit distinct bank groups.
uint64_t batch_x_pitch(const Context* c)
{
	const uint64_t vn = 16 / c->wsize;
	const uint64_t ge = (uint64_t)group_elems((int)std::min<uint64_t>(c->S, 9), (int)vn);
	uint64_t chunks = round_up(c->row_len, c->S <= 8 ? ge : vn) / vn;
	chunks += (1 + 8 - chunks % 8) % 8;
	return chunks * vn;
}

uint64_t x_row_stage_bytes(const Context* c, uint32_t mode)
{
	return (mode == kMapSubstrate ? sweep_x_sub_pitch(c->row_len, c->S, c->wsize) : batch_x_pitch(c)) * c->wsize;
}

// Largest valid rows-per-tile of a mapping under a shared-memory budget.
uint32_t x_rows_cap(const Context* c, uint32_t mode, uint64_t smem_budget)
{
	const uint64_t lanes_per_row = mode == kMapRow ? 1 : c->S;
	uint64_t r = smem_budget / x_row_stage_bytes(c, mode);
	const uint64_t cap = kLanes / lanes_per_row;
	r = std::min(r, cap);
	return (uint32_t)std::max<uint64_t>(r, 1);
}

AxisConfig default_config(const Context* c, int axis)
{
	AxisConfig a;
	if (axis == 0)
	{
		// measured on uneven batches: substrate-per-thread beats row-per-thread for every S
		a.mode = c->S <= kLanes ? kMapSubstrate : kMapRow;
		a.rows = x_rows_cap(c, a.mode, kXSmemDefault);
		return a;
	}
	uint32_t R, nc;
	box_geometry(c->n[axis], R, nc);
	a.rows = R;
	return a;
}

// Validates (and if needed repairs) a y/z chunk size: a multiple of the solver
// block, at most 256 points (the TMA box limit), at most kMaxChunks chunks.
uint32_t fit_chunk(uint64_t n, uint32_t R)
{
	R = (uint32_t)round_up(std::max<uint32_t>(R, kBlock), kBlock);
	if ((n + R - 1) / R > kMaxChunks)
		R = (uint32_t)round_up((n + kMaxChunks - 1) / kMaxChunks, kBlock);
	return std::min<uint32_t>(R, 256);
}

} // namespace
} // namespace pcg

using pcg::Context;
using pcg::fail;
using pcg::DeviceBuffer;

struct pcg_batch
{
	int device = 0;
	uint32_t* h_words = nullptr; // pinned host words for reading the error words
	pcg::DeviceBuffer d_iblocks;   // internalize: first block of each domain [N + 1]
	uint32_t internalize_blocks = 0;
	cudaEvent_t ev_block = nullptr; // blocking-sync event for host waits on the stream
	size_t wsize = 4;
	int sm_count = 0;
	std::vector<pcg_context*> ctx;
	std::vector<uint64_t> gen;
	cudaStream_t stream = nullptr;
	cudaEvent_t ev_sync = nullptr;

	std::vector<pcg::BatchDomain> h_doms;
	std::vector<CUtensorMap> h_tmaps;
	std::vector<pcg::AxisConfig> cfg[3];
	DeviceBuffer d_doms, d_tmaps, d_lists, d_counters, d_err, d_recompute, d_steps_left;
	std::vector<uint32_t> h_steps_left;
	pcg::WorkList lists[pcg::L_COUNT] {};
	uint64_t smem[3] = { 0, 0, 0 };
	unsigned grid[3] = { 0, 0, 0 };
	int max_dims = 0;
	bool built = false;
	bool any_mass_check = false; // some domain has the per-step mass check on

	std::vector<uint8_t> h_recompute, dev_recompute;
	bool dev_recompute_valid = false;

	bool use_graph = true;
	// graphs of one step with [1] and without [0] the ballot-rebuild kernels (clear,
	// locate, ballot, reduce): calls in which no domain rebuilds its ballot skip them
	cudaGraphExec_t exec[2] = { nullptr, nullptr };
	uint64_t kernels_per_step[2] = { 0, 0 };
	pcg::KernelStat graph_step[2][pcg::K_COUNT]; // launches and bytes of one replayed step
	bool step_rebuilds = true;                    // launch_step includes the rebuild kernels

	bool timing = false;
	double step_bytes[pcg::K_COUNT] = {}; // algorithmic bytes of one launch of each kernel
	// per domain: bytes of the ballot-rebuild kernels (clear, locate, ballot,
	// reduce), which only count for domains that rebuild in the current call
	std::vector<std::array<double, 4>> rebuild_bytes;
	pcg::KernelStat stats[pcg::K_COUNT];
	uint64_t launches = 0;
	struct Pending
	{
		int kid;
		cudaEvent_t a, b;
		bool shared_bytes; // add the step's shared-voxel agent bytes (timing mode)
	};
	pcg::DeviceBuffer d_shared_bytes; // timing mode: bytes of the last internalize pass
	double* h_shared_bytes = nullptr;  // pinned copy
	std::vector<Pending> pending;
	std::vector<cudaEvent_t> event_pool;

	std::vector<pcg::TuneRecord> tuned;
	bool forced[3] = { false, false, false };
	pcg::AxisConfig force[3];
};

namespace pcg {
namespace {

void free_buf(DeviceBuffer& b) { dfree(b); }

// Batch buffers come from the stream-ordered allocator on the batch's stream (all
// their users run on it), so regrouping batches never synchronises the device.
int balloc(DeviceBuffer& b, size_t bytes, cudaStream_t stream, int device)
{
	if (b.ptr && b.bytes >= bytes)
		return PCG_OK;
	dfree(b);
	if (!bytes)
		return PCG_OK;
	cudaError_t e = pool_alloc(&b.ptr, bytes, stream, device);
	if (e != cudaSuccess)
	{
		b.ptr = nullptr;
		cudaGetLastError();
		return fail(PCG_ERR_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes for a batch failed");
	}
	b.bytes = bytes;
	b.stream = stream;
	return PCG_OK;
}

Context* C(pcg_batch* b, size_t d) { return static_cast<Context*>(b->ctx[d]); }

// Host wait for the batch stream, asleep (see stream_wait in capi.cu).
cudaError_t batch_wait(pcg_batch* b)
{
	if (!b->ev_block)
	{
		cudaError_t e = cudaEventCreateWithFlags(&b->ev_block, cudaEventBlockingSync | cudaEventDisableTiming);
		if (e != cudaSuccess)
		{
			b->ev_block = nullptr;
			return e;
		}
	}
	cudaError_t e = cudaEventRecord(b->ev_block, b->stream);
	return e != cudaSuccess ? e : cudaEventSynchronize(b->ev_block);
}

// ---- descriptors

BatchDomain describe_domain(pcg_batch* b, size_t d)
{
	Context* c = C(b, d);
	BatchDomain D {};
	D.field = c->field.ptr;
	D.pitch = c->pitch;
	D.row_len = c->row_len;
	D.rows = c->rows;
	D.V = c->V;
	D.S = (uint32_t)c->S;
	D.dims = (uint32_t)c->dims;
	for (int a = 0; a < 3; a++)
	{
		D.n[a] = (uint32_t)c->n[a];
		D.coef[a] = c->coef[a].ptr;
		D.coef_len[a] = c->coef_len[a];
	}
	const AxisConfig& x = b->cfg[0][d];
	D.x_rows = x.rows;
	D.x_mode = x.mode;
	D.x_smem_pitch = x.mode == kMapSubstrate ? sweep_x_sub_pitch(c->row_len, c->S, c->wsize) : batch_x_pitch(c);
	for (int a = 1; a < c->dims; a++)
	{
		D.box_rows[a] = b->cfg[a][d].rows;
		D.boxes[a] = (uint32_t)((c->n[a] + D.box_rows[a] - 1) / D.box_rows[a]);
		const uint64_t tile_bytes = (uint64_t)D.boxes[a] * D.box_rows[a] * kLanes * c->wsize;
		D.yz_group[a] = (uint32_t)std::min<uint64_t>(kMaxGroup, std::max<uint64_t>(1, kGroupBytes / tile_bytes));
	}
	D.yz_xblocks = (c->row_len + kLanes - 1) / kLanes;
	for (int a = 0; a < c->dims; a++)
	{
		D.coef_comp_off[a] = c->coef_comp_off[a];
		D.coef_blo_off[a] = c->coef_blo_off[a];
		D.coef_head[a] = c->coef_head[a];
	}
	D.faces = make_face_args(c);
	D.dir_offsets = static_cast<const uint64_t*>(c->dir_offsets.ptr);
	D.dir_values = c->dir_values.ptr;
	D.dir_conds = static_cast<const uint8_t*>(c->dir_conds.ptr);
	D.K = c->K;
	D.bulk_mode = c->bulk_mode;
	for (int k = 0; k < 3; k++)
		D.bulk[k] = c->bulk[k].ptr;
	D.dt = c->dt;
	D.cells = make_cell_args(c);
	D.cells.err = static_cast<uint32_t*>(b->d_err.ptr);
	D.cells.list_word = 1; // the batch's per-warp ballot lists shared-voxel agents in word 1
	if (c->mass_check && c->mc_tot.ptr && c->mc_out.ptr)
	{
		D.mc_tot = static_cast<double*>(c->mc_tot.ptr);
		D.mc_out = static_cast<double*>(c->mc_out.ptr);
	}
	return D;
}

struct HostList
{
	std::vector<uint64_t> base;
	std::vector<uint32_t> dom;
};

// Units of list `id` for domain d (0 = absent), and the cost of one unit used
// to order domains (largest units first, so the last tiles handed out are small).
void list_units(pcg_batch* b, int id, size_t d, uint64_t& units, double& cost)
{
	Context* c = C(b, d);
	const BatchDomain& D = b->h_doms[d];
	units = 0;
	cost = 0;
	switch (id)
	{
	case L_X:
		units = (c->rows + D.x_rows - 1) / D.x_rows;
		cost = (double)D.x_rows * (double)c->row_len;
		break;
	case L_Y:
		if (c->dims >= 2)
			units = (D.yz_xblocks * c->n[2] + D.yz_group[1] - 1) / D.yz_group[1],
			cost = (double)c->n[1] * D.yz_group[1];
		break;
	case L_Z:
		if (c->dims >= 3)
			units = (D.yz_xblocks * c->n[1] + D.yz_group[2] - 1) / D.yz_group[2],
			cost = (double)c->n[2] * D.yz_group[2];
		break;
	case L_FACES: units = (D.faces.face_mask && c->dims == 1) ? D.faces.total * c->S : 0; break; // else fused
	case L_INTERIOR: units = c->K * c->S; break;
	case L_BULK: units = c->bulk_mode != PCG_BULK_NONE ? c->rows : 0; break;
	case L_CLEAR: units = c->A ? (c->V + kClearChunk - 1) / kClearChunk : 0; break;
	case L_AGENTS: units = c->A; break;
	}
}

HostList build_list(pcg_batch* b, int id, const std::vector<size_t>& subset)
{
	std::vector<std::pair<double, size_t>> order;
	for (size_t d : subset)
	{
		uint64_t u;
		double cost;
		list_units(b, id, d, u, cost);
		if (u)
			order.push_back({ -cost, d });
	}
	if (id <= L_Z)
		std::stable_sort(order.begin(), order.end());
	HostList h;
	uint64_t acc = 0;
	for (auto& e : order)
	{
		uint64_t u;
		double cost;
		list_units(b, id, e.second, u, cost);
		h.base.push_back(acc);
		h.dom.push_back((uint32_t)e.second);
		acc += u;
	}
	h.base.push_back(acc);
	return h;
}

// Uploads host lists into one device buffer and fills the device-side views.
int upload_lists(DeviceBuffer& buf, const std::vector<HostList>& hl, WorkList* out, cudaStream_t stream,
				 int device)
{
	// lookup hints: one entry index per block of 2^shift units, at most 2^18 blocks
	std::vector<std::vector<uint32_t>> hints(hl.size());
	std::vector<uint32_t> shifts(hl.size(), 0);
	size_t bytes = 0;
	for (size_t i = 0; i < hl.size(); i++)
	{
		const HostList& h = hl[i];
		const uint64_t total = h.base.back();
		uint32_t shift = 0;
		while ((total >> shift) > (1ull << 18))
			shift++;
		std::vector<uint32_t>& hint = hints[i];
		hint.resize((size_t)(total >> shift) + 1);
		uint32_t k = 0;
		for (size_t j = 0; j < hint.size(); j++)
		{
			const uint64_t u = (uint64_t)j << shift;
			while (k + 1 < h.dom.size() && h.base[k + 1] <= u)
				k++;
			hint[j] = k;
		}
		shifts[i] = shift;
		bytes += round_up(h.base.size() * 8, 256) + round_up(std::max<size_t>(h.dom.size(), 1) * 4, 256) +
				 round_up(hint.size() * 4, 256);
	}
	int rc = balloc(buf, bytes, stream, device);
	if (rc)
		return rc;
	std::vector<unsigned char> host(bytes, 0);
	size_t off = 0;
	for (size_t i = 0; i < hl.size(); i++)
	{
		const HostList& h = hl[i];
		memcpy(host.data() + off, h.base.data(), h.base.size() * 8);
		out[i].base = reinterpret_cast<const uint64_t*>(static_cast<unsigned char*>(buf.ptr) + off);
		off += round_up(h.base.size() * 8, 256);
		if (!h.dom.empty())
			memcpy(host.data() + off, h.dom.data(), h.dom.size() * 4);
		out[i].dom = reinterpret_cast<const uint32_t*>(static_cast<unsigned char*>(buf.ptr) + off);
		off += round_up(std::max<size_t>(h.dom.size(), 1) * 4, 256);
		memcpy(host.data() + off, hints[i].data(), hints[i].size() * 4);
		out[i].hint = reinterpret_cast<const uint32_t*>(static_cast<unsigned char*>(buf.ptr) + off);
		off += round_up(hints[i].size() * 4, 256);
		out[i].count = (uint32_t)h.dom.size();
		out[i].shift = shifts[i];
		out[i].total = h.base.back();
	}
	PCG_CUDA_TRY(cudaMemcpyAsync(buf.ptr, host.data(), bytes, cudaMemcpyHostToDevice, stream));
	PCG_CUDA_TRY(cudaStreamSynchronize(stream));
	return PCG_OK;
}

// Encodes the y/z tensor maps of domain d with its current chunk sizes.
int encode_maps(pcg_batch* b, size_t d)
{
	Context* c = C(b, d);
	for (int a = 1; a < c->dims; a++)
	{
		const int rc = encode_field_map(c, a, b->cfg[a][d].rows, &b->h_tmaps[2 * d + (a - 1)]);
		if (rc)
			return rc;
	}
	return PCG_OK;
}

int upload_domains(pcg_batch* b)
{
	const size_t N = b->ctx.size();
	b->any_mass_check = false;
	for (size_t d = 0; d < N; d++)
	{
		b->h_doms[d] = describe_domain(b, d);
		b->any_mass_check |= b->h_doms[d].mc_tot != nullptr;
	}
	// y/z: every CTA's buffer holds the batch's largest tile, so a short-line
	// domain groups its tiles up to that size (at least kGroupBytes) instead of
	// leaving most of the buffer empty
	for (int a = 1; a < 3; a++)
	{
		auto tile_bytes = [&](size_t d) {
			const BatchDomain& D = b->h_doms[d];
			return (uint64_t)D.boxes[a] * D.box_rows[a] * kLanes * b->wsize;
		};
		uint64_t cap = kGroupBytes;
		for (size_t d = 0; d < N; d++)
			if (a < C(b, d)->dims)
				cap = std::max(cap, tile_bytes(d));
		for (size_t d = 0; d < N; d++)
			if (a < C(b, d)->dims)
				b->h_doms[d].yz_group[a] =
					(uint32_t)std::min<uint64_t>(kMaxGroup, std::max<uint64_t>(1, cap / tile_bytes(d)));
	}
	int rc;
	if ((rc = balloc(b->d_doms, N * sizeof(BatchDomain), b->stream, b->device)) ||
		(rc = balloc(b->d_tmaps, N * 2 * sizeof(CUtensorMap), b->stream, b->device)))
		return rc;
	PCG_CUDA_TRY(cudaMemcpyAsync(b->d_doms.ptr, b->h_doms.data(), N * sizeof(BatchDomain), cudaMemcpyHostToDevice,
								 b->stream));
	PCG_CUDA_TRY(cudaMemcpyAsync(b->d_tmaps.ptr, b->h_tmaps.data(), N * 2 * sizeof(CUtensorMap),
								 cudaMemcpyHostToDevice, b->stream));
	PCG_CUDA_TRY(pcg::batch_wait(b));
	return PCG_OK;
}

void drop_graph(pcg_batch* b)
{
	for (auto& x : b->exec)
		if (x)
		{
			cudaGraphExecDestroy(x);
			x = nullptr;
		}
}

template <typename T>
uint64_t sweep_smem(pcg_batch* b, int axis, const std::vector<size_t>& subset)
{
	uint64_t best = 0;
	for (size_t d : subset)
	{
		Context* c = C(b, d);
		if (axis >= c->dims)
			continue;
		const BatchDomain& D = b->h_doms[d];
		if (axis == 0)
			best = std::max<uint64_t>(best, 16 + (uint64_t)D.x_rows * D.x_smem_pitch * sizeof(T));
		else
			best = std::max<uint64_t>(best, (uint64_t)D.yz_group[axis] * D.boxes[axis] * D.box_rows[axis] * kLanes *
												sizeof(T));
	}
	if (axis > 0)
		best += 128; // the tile's mbarrier
	return best;
}

template <typename T>
const void* sweep_kernel(int axis, bool mass_check)
{
	if (axis == 0)
		return mass_check ? reinterpret_cast<const void*>(batch_sweep_x_kernel<T, kMcIn | kMcOut>)
						  : reinterpret_cast<const void*>(batch_sweep_x_kernel<T, 0>);
	if (axis == 1)
		return mass_check ? reinterpret_cast<const void*>(batch_sweep_yz_kernel<T, 1, kMcOut>)
						  : reinterpret_cast<const void*>(batch_sweep_yz_kernel<T, 1, 0>);
	return mass_check ? reinterpret_cast<const void*>(batch_sweep_yz_kernel<T, 2, kMcOut>)
					  : reinterpret_cast<const void*>(batch_sweep_yz_kernel<T, 2, 0>);
}

// The dynamic shared-memory limit of a batched sweep kernel only ever grows, so
// graphs captured by other batches with larger tiles stay launchable.
std::mutex g_attr_mu;
std::map<std::pair<const void*, int>, uint64_t> g_attr_max;

int raise_smem_limit(const void* k, int device, uint64_t smem)
{
	std::lock_guard<std::mutex> lk(g_attr_mu);
	uint64_t& cur = g_attr_max[{ k, device }];
	if (smem <= cur)
		return PCG_OK;
	PCG_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	cur = smem;
	return PCG_OK;
}

// Persistent grid of a sweep launch with `smem` bytes per CTA.
template <typename T>
int sweep_grid(pcg_batch* b, int axis, uint64_t smem, uint64_t tiles, unsigned* grid)
{
	const void* k = sweep_kernel<T>(axis, b->any_mass_check);
	if (smem > kMaxSmemBytes)
		return fail(PCG_ERR_UNSUPPORTED, "a batched sweep tile exceeds shared memory");
	int rc;
	for (int mc = 0; mc < 2; mc++) // both variants: a later call may switch the check
		if ((rc = raise_smem_limit(sweep_kernel<T>(axis, mc != 0), b->device, smem)))
			return rc;
	int per_sm = 0;
	PCG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kLanes, smem));
	if (per_sm < 1)
		return fail(PCG_ERR_UNSUPPORTED, "a batched sweep tile does not fit on an SM");
	uint64_t g = (uint64_t)per_sm * (uint64_t)b->sm_count;
	*grid = (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(g, tiles));
	return PCG_OK;
}

template <typename T>
int build_t(pcg_batch* b)
{
	const size_t N = b->ctx.size();
	std::vector<size_t> all(N);
	std::iota(all.begin(), all.end(), 0);
	int rc;
	for (size_t d = 0; d < N; d++)
		if ((rc = encode_maps(b, d)))
			return rc;
	if ((rc = upload_domains(b)))
		return rc;
	std::vector<HostList> hl;
	for (int id = 0; id < L_COUNT; id++)
		hl.push_back(build_list(b, id, all));
	if ((rc = upload_lists(b->d_lists, hl, b->lists, b->stream, b->device)))
		return rc;
	for (int axis = 0; axis < 3; axis++)
	{
		b->smem[axis] = 0;
		if (b->lists[axis].total == 0)
			continue;
		b->smem[axis] = sweep_smem<T>(b, axis, all);
		if ((rc = sweep_grid<T>(b, axis, b->smem[axis], b->lists[axis].total, &b->grid[axis])))
			return rc;
	}
	// internalize blocks per domain in proportion to its agents (those in shared
	// voxels are only known on the device): block0[d] .. block0[d+1]
	{
		std::vector<uint32_t> block0(N + 1, 0);
		double total = 0;
		for (size_t d = 0; d < N; d++)
			total += C(b, d)->compute_internalized ? (double)C(b, d)->A : 0.0;
		const double G = 8.0 * std::max(b->sm_count, 1);
		for (size_t d = 0; d < N; d++)
		{
			const Context* c = C(b, d);
			const double w = c->compute_internalized ? (double)c->A : 0.0;
			const uint32_t blocks = w > 0 ? (uint32_t)std::max(1.0, std::floor(G * w / total)) : 0u;
			block0[d + 1] = block0[d] + blocks;
		}
		b->internalize_blocks = block0[N];
		if ((rc = balloc(b->d_iblocks, (N + 1) * sizeof(uint32_t), b->stream, b->device)))
			return rc;
		PCG_CUDA_TRY(cudaMemcpyAsync(b->d_iblocks.ptr, block0.data(), (N + 1) * sizeof(uint32_t),
									 cudaMemcpyHostToDevice, b->stream));
		PCG_CUDA_TRY(batch_wait(b));
	}
	// algorithmic bytes per launch, with the single-domain launchers' per-item counts
	std::fill(b->step_bytes, b->step_bytes + K_COUNT, 0.0);
	b->rebuild_bytes.assign(N, { 0.0, 0.0, 0.0, 0.0 });
	const double w = (double)sizeof(T);
	for (size_t d = 0; d < N; d++)
	{
		const Context* c = C(b, d);
		const double V = (double)c->V, S = (double)c->S, A = (double)c->A;
		for (int a = 0; a < c->dims; a++)
			b->step_bytes[K_SWEEP_X + a] += 2.0 * V * S * w;
		const FaceArgs& f = b->h_doms[d].faces;
		if (f.face_mask && c->dims == 1) // otherwise written by the last sweep
			b->step_bytes[K_DIRICHLET_FACES] += (double)f.total * S * w;
		b->step_bytes[K_DIRICHLET_INTERIOR] += (double)c->K * (8 + S * (2 * w + 1));
		if (c->bulk_mode != PCG_BULK_NONE)
			b->step_bytes[K_BULK] += V * S * w * (c->bulk_mode == PCG_BULK_PER_VOXEL ? 5.0 : 2.0);
		if (b->h_doms[d].mc_tot)
			b->step_bytes[K_MASS_CHECK] += 6 * S * 8;
		if (c->A)
		{
			b->rebuild_bytes[d] = { 4.0 * V, A * (8.0 * c->dims + 1 + 5 * S * 8 + 8 + 6 * S * w + 4), A * 12,
									A * (8 + 6 * S * w) };
			b->step_bytes[K_CELLS_APPLY] += A * (5 + 5 * S * w + (c->compute_internalized ? 16 * S : 0));
			// internalize: counted per agent of a shared voxel in timing mode (the
			// lists' lengths are on the device), not in replayed steps
		}
	}
	b->built = true;
	drop_graph(b);
	return PCG_OK;
}

// ---- launches

cudaEvent_t get_event(pcg_batch* b)
{
	if (!b->event_pool.empty())
	{
		cudaEvent_t e = b->event_pool.back();
		b->event_pool.pop_back();
		return e;
	}
	cudaEvent_t e = nullptr;
	cudaEventCreate(&e);
	return e;
}

struct LaunchScope
{
	pcg_batch* b;
	int kid;
	double bytes;
	cudaEvent_t a = nullptr;
	LaunchScope(pcg_batch* b_, int kid_, double bytes_) : b(b_), kid(kid_), bytes(bytes_)
	{
		b->launches++;
		b->stats[kid].launches++;
		b->stats[kid].bytes += bytes;
		if (b->timing)
		{
			a = get_event(b);
			cudaEventRecord(a, b->stream);
		}
	}
	~LaunchScope()
	{
		if (a)
		{
			cudaEvent_t e = get_event(b);
			cudaEventRecord(e, b->stream);
			b->pending.push_back({ kid, a, e, kid == K_CELLS_INTERNALIZE });
		}
	}
};

void collect(pcg_batch* b)
{
	for (auto& p : b->pending)
	{
		float ms = 0;
		if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess)
			b->stats[p.kid].total_ms += ms;
		if (p.shared_bytes && b->h_shared_bytes)
			b->stats[p.kid].bytes += *b->h_shared_bytes;
		b->event_pool.push_back(p.a);
		b->event_pool.push_back(p.b);
	}
	b->pending.clear();
	cudaGetLastError();
}

BatchArgs args_for(pcg_batch* b, int list, int counter)
{
	BatchArgs a {};
	a.doms = static_cast<const BatchDomain*>(b->d_doms.ptr);
	a.tmaps = static_cast<const CUtensorMap*>(b->d_tmaps.ptr);
	a.list = b->lists[list];
	a.counter = static_cast<uint32_t*>(b->d_counters.ptr) + counter;
	a.err = static_cast<uint32_t*>(b->d_err.ptr);
	a.recompute = static_cast<const uint8_t*>(b->d_recompute.ptr);
	a.steps_left = static_cast<uint32_t*>(b->d_steps_left.ptr);
	return a;
}

unsigned flat_grid(pcg_batch* b, uint64_t work, unsigned block)
{
	uint64_t g = (work + block - 1) / block;
	const uint64_t cap = (uint64_t)b->sm_count * 16;
	return (unsigned)std::max<uint64_t>(1, std::min(g, cap));
}

// Launches one sweep axis over a work list (used by the step and by the tuner).
template <typename T>
int launch_sweep(pcg_batch* b, int axis, const BatchArgs& a, unsigned grid, uint64_t smem, double bytes)
{
	LaunchScope s(b, axis == 0 ? K_SWEEP_X : axis == 1 ? K_SWEEP_Y : K_SWEEP_Z, bytes);
	const bool mc = b->any_mass_check;
	if (axis == 0)
		(mc ? batch_sweep_x_kernel<T, kMcIn | kMcOut> : batch_sweep_x_kernel<T, 0>)<<<grid, kLanes, smem, b->stream>>>(a);
	else if (axis == 1)
		(mc ? batch_sweep_yz_kernel<T, 1, kMcOut>
			: batch_sweep_yz_kernel<T, 1, 0>)<<<grid, kLanes, smem, b->stream>>>(a);
	else
		(mc ? batch_sweep_yz_kernel<T, 2, kMcOut>
			: batch_sweep_yz_kernel<T, 2, 0>)<<<grid, kLanes, smem, b->stream>>>(a);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

// One step of every domain, in the reference's phase order.
template <typename T>
int launch_step(pcg_batch* b)
{
	const double* sb = b->step_bytes;
	PCG_CUDA_TRY(cudaMemsetAsync(b->d_counters.ptr, 0, 4 * sizeof(uint32_t), b->stream));
	int rc;
	for (int axis = 0; axis < 3; axis++)
		if (b->lists[axis].total && (rc = launch_sweep<T>(b, axis, args_for(b, axis, axis), b->grid[axis],
														   b->smem[axis], sb[K_SWEEP_X + axis])))
			return rc;
	if (b->any_mass_check)
	{
		LaunchScope s(b, K_MASS_CHECK, sb[K_MASS_CHECK]);
		const uint32_t N = (uint32_t)b->ctx.size();
		batch_mass_finish_kernel<<<std::min<uint32_t>(N, 1024), 32, 0, b->stream>>>(
			static_cast<const BatchDomain*>(b->d_doms.ptr), static_cast<const uint32_t*>(b->d_steps_left.ptr), N);
		PCG_CUDA_TRY(cudaGetLastError());
	}
	if (b->lists[L_FACES].total)
	{
		LaunchScope s(b, K_DIRICHLET_FACES, sb[K_DIRICHLET_FACES]);
		batch_faces_kernel<T><<<flat_grid(b, b->lists[L_FACES].total, 256), 256, 0, b->stream>>>(
			args_for(b, L_FACES, 3));
		PCG_CUDA_TRY(cudaGetLastError());
	}
	if (b->lists[L_INTERIOR].total)
	{
		LaunchScope s(b, K_DIRICHLET_INTERIOR, sb[K_DIRICHLET_INTERIOR]);
		batch_interior_kernel<T><<<flat_grid(b, b->lists[L_INTERIOR].total, 256), 256, 0, b->stream>>>(
			args_for(b, L_INTERIOR, 3));
		PCG_CUDA_TRY(cudaGetLastError());
	}
	if (b->lists[L_BULK].total)
	{
		LaunchScope s(b, K_BULK, sb[K_BULK]);
		batch_bulk_kernel<T><<<flat_grid(b, b->lists[L_BULK].total * 32, 256), 256, 0, b->stream>>>(
			args_for(b, L_BULK, 3));
		PCG_CUDA_TRY(cudaGetLastError());
	}
	const uint64_t A = b->lists[L_AGENTS].total;
	if (A)
	{
		const unsigned g = (unsigned)((A + 255) / 256);
		if (b->step_rebuilds)
		{
			{
				LaunchScope s(b, K_CELLS_CLEAR, sb[K_CELLS_CLEAR]);
				batch_clear_counts_kernel<<<flat_grid(b, b->lists[L_CLEAR].total * 32, 256), 256, 0, b->stream>>>(
					args_for(b, L_CLEAR, 3));
				PCG_CUDA_TRY(cudaGetLastError());
			}
			{
				LaunchScope s(b, K_CELLS_LOCATE, sb[K_CELLS_LOCATE]);
				batch_cells_locate_kernel<T><<<g, 256, 0, b->stream>>>(args_for(b, L_AGENTS, 3));
				PCG_CUDA_TRY(cudaGetLastError());
			}
			{
				LaunchScope s(b, K_CELLS_BALLOT, sb[K_CELLS_BALLOT]);
				batch_cells_ballot_kernel<<<g, 256, 0, b->stream>>>(args_for(b, L_AGENTS, 3));
				PCG_CUDA_TRY(cudaGetLastError());
			}
			{
				LaunchScope s(b, K_CELLS_REDUCE, sb[K_CELLS_REDUCE]);
				batch_cells_reduce_kernel<T><<<g, 256, 0, b->stream>>>(args_for(b, L_AGENTS, 3));
				PCG_CUDA_TRY(cudaGetLastError());
			}
		}
		{
			LaunchScope s(b, K_CELLS_APPLY, sb[K_CELLS_APPLY]);
			batch_cells_apply_kernel<T><<<g, 256, 0, b->stream>>>(args_for(b, L_AGENTS, 3));
			PCG_CUDA_TRY(cudaGetLastError());
		}
		{
			LaunchScope s(b, K_CELLS_INTERNALIZE, sb[K_CELLS_INTERNALIZE]);
			const uint32_t ndom = (uint32_t)b->ctx.size();
			batch_cells_internalize_kernel<T><<<std::max(b->internalize_blocks, 1u), 256, 0, b->stream>>>(
				args_for(b, L_AGENTS, 3), static_cast<const uint32_t*>(b->d_iblocks.ptr), ndom);
			PCG_CUDA_TRY(cudaGetLastError());
		}
		if (b->timing) // the internalize pass's bytes, once the lists' lengths are known
		{
			if (!b->h_shared_bytes)
				b->h_shared_bytes = reinterpret_cast<double*>(pinned_words_get());
			if (!b->h_shared_bytes)
				return fail(PCG_ERR_NOMEM, "pinned host memory for the internalize byte count");
			const int rc2 = balloc(b->d_shared_bytes, sizeof(double), b->stream, b->device);
			if (rc2)
				return rc2;
			batch_shared_bytes_kernel<<<1, 256, 0, b->stream>>>(
				static_cast<const BatchDomain*>(b->d_doms.ptr), static_cast<const uint32_t*>(b->d_steps_left.ptr),
				(uint32_t)b->ctx.size(), (uint32_t)sizeof(T), static_cast<double*>(b->d_shared_bytes.ptr));
			PCG_CUDA_TRY(cudaMemcpyAsync(b->h_shared_bytes, b->d_shared_bytes.ptr, sizeof(double),
										 cudaMemcpyDeviceToHost, b->stream));
		}
	}
	const uint32_t N = (uint32_t)b->ctx.size();
	batch_count_step_kernel<<<(N + 255) / 256, 256, 0, b->stream>>>(static_cast<uint32_t*>(b->d_steps_left.ptr), N);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

int step(pcg_batch* b) { return b->wsize == 4 ? launch_step<float>(b) : launch_step<double>(b); }

int capture(pcg_batch* b, int rebuilds)
{
	cudaGraph_t g = nullptr;
	const uint64_t before = b->launches;
	KernelStat stats_before[K_COUNT];
	std::copy(b->stats, b->stats + K_COUNT, stats_before);
	PCG_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
	const bool timing = b->timing;
	b->timing = false;
	b->step_rebuilds = rebuilds != 0;
	int rc = step(b);
	b->timing = timing;
	cudaError_t e = cudaStreamEndCapture(b->stream, &g);
	if (rc)
	{
		if (g)
			cudaGraphDestroy(g);
		return rc;
	}
	if (e != cudaSuccess)
		return fail(PCG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
	e = cudaGraphInstantiate(&b->exec[rebuilds], g, 0);
	cudaGraphDestroy(g);
	if (e != cudaSuccess)
	{
		b->exec[rebuilds] = nullptr;
		return fail(PCG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
	}
	// capture counted the step's kernels once without running them: keep the
	// per-step counts and add them on every replay instead
	b->kernels_per_step[rebuilds] = b->launches - before;
	b->launches = before;
	for (int k = 0; k < K_COUNT; k++)
	{
		b->graph_step[rebuilds][k].launches = b->stats[k].launches - stats_before[k].launches;
		b->graph_step[rebuilds][k].bytes = b->stats[k].bytes - stats_before[k].bytes;
		b->stats[k] = stats_before[k];
	}
	return PCG_OK;
}

// Rebuilds descriptors when any context changed since the last build.
int refresh(pcg_batch* b)
{
	bool changed = !b->built;
	for (size_t d = 0; d < b->ctx.size(); d++)
	{
		Context* c = C(b, d);
		int rc = initialize_context(c);
		if (rc)
			return rc;
		if (c->generation != b->gen[d])
			changed = true;
	}
	if (!changed)
		return PCG_OK;
	for (size_t d = 0; d < b->ctx.size(); d++)
	{
		Context* c = C(b, d);
		b->gen[d] = c->generation;
		for (int a = 0; a < c->dims; a++)
		{
			std::lock_guard<std::mutex> lk(g_tune_mu);
			auto it = g_tuned.find(bucket_key(a, c->wsize, c->S, c->n[a]));
			AxisConfig cfg = it != g_tuned.end() ? it->second : default_config(c, a);
			if (b->forced[a])
			{
				const AxisConfig dflt = default_config(c, a);
				cfg = b->force[a];
				if (a == 0 && (cfg.mode != kMapSubstrate || c->S > kLanes))
					cfg.mode = kMapRow;
				if (cfg.rows == 0)
					cfg.rows = a == 0 ? x_rows_cap(c, cfg.mode, kXSmemDefault) : dflt.rows;
			}
			if (a == 0)
				cfg.rows = std::min(cfg.rows, x_rows_cap(c, cfg.mode, kMaxSmemBytes - 16));
			else
				cfg.rows = fit_chunk(c->n[a], cfg.rows);
			b->cfg[a][d] = cfg;
		}
	}
	return b->wsize == 4 ? build_t<float>(b) : build_t<double>(b);
}

// The distinct streams of the batch's contexts, other than the batch's own.
std::vector<cudaStream_t> context_streams(pcg_batch* b)
{
	std::vector<cudaStream_t> out;
	out.reserve(b->ctx.size());
	for (size_t d = 0; d < b->ctx.size(); d++)
		if (C(b, d)->stream != b->stream)
			out.push_back(C(b, d)->stream);
	std::sort(out.begin(), out.end());
	out.erase(std::unique(out.begin(), out.end()), out.end());
	return out;
}

int sync_in(pcg_batch* b)
{
	for (cudaStream_t s : context_streams(b))
	{
		// a stream with nothing left to run needs no wait (hundreds of served
		// requests: one query instead of an event record and a wait each)
		if (cudaStreamQuery(s) == cudaSuccess)
			continue;
		PCG_CUDA_TRY(cudaEventRecord(b->ev_sync, s));
		PCG_CUDA_TRY(cudaStreamWaitEvent(b->stream, b->ev_sync, 0));
	}
	return PCG_OK;
}

int sync_out(pcg_batch* b)
{
	PCG_CUDA_TRY(cudaEventRecord(b->ev_sync, b->stream));
	for (cudaStream_t s : context_streams(b))
		PCG_CUDA_TRY(cudaStreamWaitEvent(s, b->ev_sync, 0));
	return PCG_OK;
}

int upload_recompute(pcg_batch* b)
{
	const size_t N = b->ctx.size();
	for (size_t d = 0; d < N; d++)
		b->h_recompute[d] = C(b, d)->recompute_cells || C(b, d)->ballot_kind != 2 ? 1 : 0;
	static const int rebuild_kernels[4] = { K_CELLS_CLEAR, K_CELLS_LOCATE, K_CELLS_BALLOT, K_CELLS_REDUCE };
	for (int k = 0; k < 4; k++)
	{
		double sum = 0;
		for (size_t d = 0; d < N; d++)
			sum += b->h_recompute[d] ? b->rebuild_bytes[d][k] : 0.0;
		b->step_bytes[rebuild_kernels[k]] = sum;
		b->graph_step[1][rebuild_kernels[k]].bytes = sum;
	}
	if (b->dev_recompute_valid && b->dev_recompute == b->h_recompute)
		return PCG_OK;
	PCG_CUDA_TRY(cudaMemcpyAsync(b->d_recompute.ptr, b->h_recompute.data(), N, cudaMemcpyHostToDevice, b->stream));
	PCG_CUDA_TRY(pcg::batch_wait(b)); // the host buffer is reused by the next call
	b->dev_recompute = b->h_recompute;
	b->dev_recompute_valid = true;
	return PCG_OK;
}

int check_batch(pcg_batch* b)
{
	cudaError_t e = pcg::batch_wait(b);
	if (e != cudaSuccess)
		return fail(PCG_ERR_CUDA, std::string("batch stream synchronise: ") + cudaGetErrorString(e));
	collect(b);
	if (!b->h_words && !(b->h_words = pinned_words_get()))
		return fail(PCG_ERR_NOMEM, "pinned host memory for the batch error words");
	PCG_CUDA_TRY(cudaMemcpyAsync(b->h_words, b->d_err.ptr, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, b->stream));
	PCG_CUDA_TRY(pcg::batch_wait(b));
	const uint32_t word[2] = { b->h_words[0], b->h_words[1] };
	if (word[0])
	{
		uint32_t* d = static_cast<uint32_t*>(b->d_err.ptr);
		PCG_CUDA_TRY(cudaMemsetAsync(d, 0, sizeof(uint32_t), b->stream));
		PCG_CUDA_TRY(cudaMemsetAsync(d + 1, 0xff, sizeof(uint32_t), b->stream));
		std::string msg = device_error_text(word[0]);
		if (word[1] != 0xffffffffu)
			msg += " (batch domain " + std::to_string(word[1]) + ")";
		return fail(PCG_ERR_DEVICE, msg);
	}
	return PCG_OK;
}

// ---- autotuner

template <typename T>
int time_axis(pcg_batch* b, int axis, const std::vector<size_t>& subset, double* us)
{
	int rc;
	std::vector<HostList> hl { build_list(b, axis, subset) };
	DeviceBuffer lbuf;
	WorkList wl {};
	if ((rc = upload_lists(lbuf, hl, &wl, b->stream, b->device)))
		return rc;
	const uint64_t smem = sweep_smem<T>(b, axis, subset);
	unsigned grid = 0;
	if ((rc = sweep_grid<T>(b, axis, smem, wl.total, &grid)))
	{
		dfree(lbuf);
		return rc;
	}
	BatchArgs a = args_for(b, axis, axis);
	a.list = wl;
	// every domain takes part in the timed launches
	cudaMemsetAsync(b->d_steps_left.ptr, 0x01, b->ctx.size() * sizeof(uint32_t), b->stream);
	cudaEvent_t e0, e1;
	cudaEventCreate(&e0);
	cudaEventCreate(&e1);
	const int warm = 2, reps = 5;
	const bool timing = b->timing;
	b->timing = false;
	for (int r = 0; r < warm + reps && !rc; r++)
	{
		if (r == warm)
			cudaEventRecord(e0, b->stream);
		cudaMemsetAsync(a.counter, 0, sizeof(uint32_t), b->stream);
		rc = launch_sweep<T>(b, axis, a, grid, smem, 0);
	}
	b->timing = timing;
	cudaEventRecord(e1, b->stream);
	cudaError_t e = cudaEventSynchronize(e1);
	float ms = 0;
	cudaEventElapsedTime(&ms, e0, e1);
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	dfree(lbuf);
	if (rc)
		return rc;
	if (e != cudaSuccess)
		return fail(PCG_ERR_CUDA, std::string("autotune launch: ") + cudaGetErrorString(e));
	*us = 1000.0 * ms / reps;
	return PCG_OK;
}

std::vector<AxisConfig> candidates(const Context* c, int axis)
{
	std::vector<AxisConfig> out;
	auto add = [&](AxisConfig a) {
		if (std::find(out.begin(), out.end(), a) == out.end())
			out.push_back(a);
	};
	if (axis == 0)
	{
		if (c->S <= kLanes)
			for (uint64_t budget : { (uint64_t)16384, (uint64_t)32768, (uint64_t)57344 })
				add({ kMapSubstrate, x_rows_cap(c, kMapSubstrate, budget) });
		for (uint64_t budget : { (uint64_t)32768, (uint64_t)57344 })
			add({ kMapRow, x_rows_cap(c, kMapRow, budget) });
		return out;
	}
	const uint64_t n = c->n[axis];
	for (uint32_t R : { 16u, 32u, 64u, 128u })
		if (R < n)
			add({ kMapColumn, fit_chunk(n, R) });
	add({ kMapColumn, fit_chunk(n, (uint32_t)round_up(n, kBlock)) }); // fewest boxes per line
	return out;
}

template <typename T>
int autotune_t(pcg_batch* b)
{
	int rc = refresh(b);
	if (rc)
		return rc;
	const size_t N = b->ctx.size();
	// buckets still unknown to the process-wide cache
	std::map<uint64_t, std::vector<size_t>> todo[3];
	for (size_t d = 0; d < N; d++)
	{
		Context* c = C(b, d);
		for (int a = 0; a < c->dims; a++)
		{
			const uint64_t key = bucket_key(a, c->wsize, c->S, c->n[a]);
			std::lock_guard<std::mutex> lk(g_tune_mu);
			if (!g_tuned.count(key))
				todo[a][key].push_back(d);
		}
	}
	if (todo[0].empty() && todo[1].empty() && todo[2].empty())
		return PCG_OK;
	// trial launches are not part of the batch's record
	KernelStat stats_before[K_COUNT];
	std::copy(b->stats, b->stats + K_COUNT, stats_before);
	const uint64_t launches_before = b->launches;
	// the trials sweep the fields: save them and put them back afterwards
	std::vector<size_t> off(N + 1, 0);
	for (size_t d = 0; d < N; d++)
		off[d + 1] = off[d] + round_up(C(b, d)->rows * C(b, d)->pitch * b->wsize, 256);
	DeviceBuffer save;
	if ((rc = balloc(save, off[N], b->stream, b->device)))
		return fail(PCG_ERR_NOMEM, "autotune needs a copy of the batch's fields and could not allocate it");
	for (size_t d = 0; d < N; d++)
		cudaMemcpyAsync(static_cast<char*>(save.ptr) + off[d], C(b, d)->field.ptr,
						C(b, d)->rows * C(b, d)->pitch * b->wsize, cudaMemcpyDeviceToDevice, b->stream);
	// In context: a candidate is timed on the whole axis launch (every domain of the
	// batch, the other buckets at their current choice), so that what is measured
	// is the bucket's effect on the launch the batch will run, not the latency of a
	// tiny launch.  Buckets are tuned in decreasing order of work; those below
	// kTuneShare of the axis keep the default mapping (their effect is below the
	// timing noise) and are not cached.
	for (int axis = 0; axis < 3 && !rc; axis++)
	{
		if (todo[axis].empty())
			continue;
		std::vector<size_t> axis_doms;
		double axis_work = 0;
		for (size_t d = 0; d < N; d++)
			if (axis < C(b, d)->dims)
			{
				axis_doms.push_back(d);
				axis_work += (double)C(b, d)->V * (double)C(b, d)->S;
			}
		std::vector<std::pair<double, uint64_t>> order;
		for (auto& kv : todo[axis])
		{
			double w = 0;
			for (size_t d : kv.second)
				w += (double)C(b, d)->V * (double)C(b, d)->S;
			order.push_back({ -w, kv.first });
		}
		std::sort(order.begin(), order.end());
		for (const auto& ow : order)
		{
			const std::vector<size_t>& dom = todo[axis][ow.second];
			if (-ow.first < kTuneShare * axis_work)
				continue;
			Context* c0 = C(b, dom[0]);
			TuneRecord rec {};
			rec.axis = axis;
			rec.n_bucket = bucket_of(c0->n[axis]);
			rec.S = axis == 0 ? c0->S : 0;
			rec.domains = dom.size();
			rec.best_us = 1e300;
			rec.share = -ow.first / axis_work;
			for (const AxisConfig& cand : candidates(c0, axis))
			{
				for (size_t d : dom)
				{
					AxisConfig cf = cand;
					Context* c = C(b, d);
					cf.rows = axis == 0 ? std::min(cf.rows, x_rows_cap(c, cf.mode, kMaxSmemBytes - 16))
										: fit_chunk(c->n[axis], cf.rows);
					b->cfg[axis][d] = cf;
					if (axis > 0 && (rc = encode_maps(b, d)))
						break;
				}
				if (rc || (rc = upload_domains(b)))
					break;
				double us = 0;
				if ((rc = time_axis<T>(b, axis, axis_doms, &us)))
					break;
				rec.tried.push_back({ cand, us });
				if (us < rec.best_us)
				{
					rec.best_us = us;
					rec.best = cand;
				}
			}
			if (rc)
				break;
			for (size_t d : dom) // keep the winner while the next buckets are timed
			{
				AxisConfig cf = rec.best;
				Context* c = C(b, d);
				cf.rows = axis == 0 ? std::min(cf.rows, x_rows_cap(c, cf.mode, kMaxSmemBytes - 16))
									: fit_chunk(c->n[axis], cf.rows);
				b->cfg[axis][d] = cf;
				if (axis > 0 && (rc = encode_maps(b, d)))
					break;
			}
			if (rc)
				break;
			{
				std::lock_guard<std::mutex> lk(g_tune_mu);
				g_tuned[ow.second] = rec.best;
			}
			b->tuned.push_back(rec);
		}
	}
	for (size_t d = 0; d < N; d++)
		cudaMemcpyAsync(C(b, d)->field.ptr, static_cast<char*>(save.ptr) + off[d],
						C(b, d)->rows * C(b, d)->pitch * b->wsize, cudaMemcpyDeviceToDevice, b->stream);
	cudaError_t e = pcg::batch_wait(b);
	dfree(save);
	std::copy(stats_before, stats_before + K_COUNT, b->stats);
	b->launches = launches_before;
	if (rc)
		return rc;
	if (e != cudaSuccess)
		return fail(PCG_ERR_CUDA, std::string("autotune: ") + cudaGetErrorString(e));
	if ((rc = check_batch(b)))
		return rc;
	b->built = false; // rebuild with the tuned choices
	return refresh(b);
}

std::string describe(pcg_batch* b)
{
	std::string s = "{\"domains\": " + std::to_string(b->ctx.size()) + ", \"buckets\": [";
	bool first = true;
	for (const TuneRecord& r : b->tuned)
	{
		s += first ? "" : ", ";
		first = false;
		auto cfg_txt = [&](const AxisConfig& a) {
			if (r.axis == 0)
				return std::string("{\"mapping\": \"") + (a.mode == kMapRow ? "row-per-thread" : "substrate-per-thread") +
					   "\", \"rows_per_tile\": " + std::to_string(a.rows) + "}";
			return std::string("{\"mapping\": \"column-per-lane\", \"box_points\": ") + std::to_string(a.rows) + "}";
		};
		s += "{\"axis\": " + std::to_string(r.axis) + ", \"share\": " + std::to_string(r.share) +
			 ", \"line_bucket\": " + std::to_string(r.n_bucket) +
			 ", \"substrates\": " + std::to_string(r.S) + ", \"domains\": " + std::to_string(r.domains) +
			 ", \"choice\": " + cfg_txt(r.best) + ", \"us\": " + std::to_string(r.best_us) + ", \"tried\": [";
		for (size_t i = 0; i < r.tried.size(); i++)
			s += (i ? ", " : "") + std::string("[") + cfg_txt(r.tried[i].first) + ", " +
				 std::to_string(r.tried[i].second) + "]";
		s += "]}";
	}
	s += "]}";
	return s;
}

} // namespace
} // namespace pcg

#define BATCH_CHECK(b)                                                                                       \
	do                                                                                                       \
	{                                                                                                        \
		if (!(b))                                                                                            \
			return fail(PCG_ERR_INVALID, "null batch");                                                      \
	} while (0)

extern "C" {

int pcg_batch_create(pcg_batch** out, pcg_context* const* contexts, uint64_t count)
{
	if (!out || (!contexts && count))
		return fail(PCG_ERR_INVALID, "null argument");
	*out = nullptr;
	if (count == 0)
		return fail(PCG_ERR_INVALID, "a batch needs at least one context");
	if (count >= 0xffffffffull)
		return fail(PCG_ERR_UNSUPPORTED, "too many contexts for one batch");
	auto* b = new pcg_batch();
	b->ctx.assign(contexts, contexts + count);
	const Context* c0 = b->ctx[0];
	if (!c0)
	{
		delete b;
		return fail(PCG_ERR_INVALID, "null context in batch");
	}
	b->device = c0->device;
	b->wsize = c0->wsize;
	b->sm_count = c0->sm_count;
	for (uint64_t i = 0; i < count; i++)
	{
		const Context* c = b->ctx[i];
		if (!c || c->device != b->device || c->wsize != b->wsize)
		{
			delete b;
			return fail(PCG_ERR_INVALID, "batched contexts must share one device and one precision");
		}
		for (uint64_t j = 0; j < i; j++)
			if (b->ctx[j] == b->ctx[i])
			{
				delete b;
				return fail(PCG_ERR_INVALID, "a context appears twice in the batch");
			}
		b->max_dims = std::max(b->max_dims, c->dims);
	}
	pcg::DeviceGuard g(b->device);
	auto bail = [&](int rc) {
		pcg_batch_destroy(b);
		return rc;
	};
	if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
		cudaEventCreateWithFlags(&b->ev_sync, cudaEventDisableTiming) != cudaSuccess)
		return bail(fail(PCG_ERR_CUDA, "could not create the batch stream"));
	b->gen.assign(count, ~0ull);
	b->h_doms.resize(count);
	b->h_tmaps.resize(2 * count);
	for (auto& c : b->cfg)
		c.assign(count, pcg::AxisConfig {});
	b->h_recompute.assign(count, 0);
	int rc;
	if ((rc = pcg::balloc(b->d_counters, 16 * sizeof(uint32_t), b->stream, b->device)) ||
		(rc = pcg::balloc(b->d_err, 2 * sizeof(uint32_t), b->stream, b->device)) ||
		(rc = pcg::balloc(b->d_recompute, count, b->stream, b->device)) ||
		(rc = pcg::balloc(b->d_steps_left, count * sizeof(uint32_t), b->stream, b->device)))
		return bail(rc);
	b->h_steps_left.assign(count, 0);
	const uint32_t reset[2] = { 0, 0xffffffffu };
	if (cudaMemcpyAsync(b->d_err.ptr, reset, sizeof(reset), cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
		pcg::batch_wait(b) != cudaSuccess)
		return bail(fail(PCG_ERR_CUDA, "could not clear the batch error word"));
	if ((rc = pcg::refresh(b)))
		return bail(rc);
	*out = b;
	return PCG_OK;
}

int pcg_batch_destroy(pcg_batch* b)
{
	if (!b)
		return PCG_OK;
	pcg::DeviceGuard g(b->device);
	if (b->stream)
		pcg::batch_wait(b);
	pcg::drop_graph(b);
	pcg::collect(b);
	for (cudaEvent_t e : b->event_pool)
		cudaEventDestroy(e);
	DeviceBuffer* bufs[] = { &b->d_doms,	 &b->d_tmaps,	  &b->d_lists,		&b->d_counters,
							 &b->d_err, &b->d_recompute, &b->d_steps_left, &b->d_iblocks, &b->d_shared_bytes };
	for (DeviceBuffer* x : bufs)
		pcg::free_buf(*x);
	if (b->ev_sync)
		cudaEventDestroy(b->ev_sync);
	if (b->stream)
		cudaStreamDestroy(b->stream);
	pcg::pinned_words_put(b->h_words);
	pcg::pinned_words_put(reinterpret_cast<uint32_t*>(b->h_shared_bytes));
	if (b->ev_block)
		cudaEventDestroy(b->ev_block);
	delete b;
	return PCG_OK;
}

int pcg_batch_solve(pcg_batch* b, uint64_t iterations)
{
	return pcg_batch_solve_budgets(b, iterations, nullptr);
}

int pcg_batch_solve_budgets(pcg_batch* b, uint64_t iterations, const uint64_t* budgets)
{
	BATCH_CHECK(b);
	if (iterations == 0)
		return PCG_OK;
	if (iterations >= 0xffffffffull)
		return fail(PCG_ERR_UNSUPPORTED, "at most 2^32-2 iterations per call");
	pcg::DeviceGuard g(b->device);
	int rc;
	if ((rc = pcg::refresh(b)) || (rc = pcg::sync_in(b)) || (rc = pcg::upload_recompute(b)))
		return rc;
	for (size_t d = 0; d < b->ctx.size(); d++)
		b->h_steps_left[d] = (uint32_t)(budgets ? std::min(budgets[d], iterations) : iterations);
	PCG_CUDA_TRY(cudaMemcpyAsync(b->d_steps_left.ptr, b->h_steps_left.data(), b->ctx.size() * sizeof(uint32_t),
								 cudaMemcpyHostToDevice, b->stream));
	// pageable source: the copy is staged before the call returns, so the next call may rewrite it
	// the ballot-rebuild kernels run only in calls where some stepping domain rebuilds
	int rebuilds = 0;
	for (size_t d = 0; d < b->ctx.size(); d++)
		rebuilds |= b->h_recompute[d] && b->h_steps_left[d] > 0;
	b->step_rebuilds = rebuilds != 0;
	const bool graph = b->use_graph && !b->timing;
	if (graph && !b->exec[rebuilds] && (rc = pcg::capture(b, rebuilds)))
		return rc;
	for (uint64_t it = 0; it < iterations; it++)
	{
		if (graph)
		{
			cudaError_t e = cudaGraphLaunch(b->exec[rebuilds], b->stream);
			if (e != cudaSuccess)
				return fail(PCG_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(e));
			b->launches += b->kernels_per_step[rebuilds];
			for (int k = 0; k < pcg::K_COUNT; k++)
			{
				b->stats[k].launches += b->graph_step[rebuilds][k].launches;
				b->stats[k].bytes += b->graph_step[rebuilds][k].bytes;
			}
		}
		else if ((rc = pcg::step(b)))
			return rc;
	}
	for (size_t d = 0; d < b->ctx.size(); d++)
	{
		Context* c = static_cast<Context*>(b->ctx[d]);
		if (!budgets || budgets[d] > 0)
		{
			c->recompute_cells = false;
			c->ballot_kind = 2; // the roles and lists are this batch's (rebuilt above if they were not)
		}
		if (b->h_doms[d].mc_tot)
			c->mass_checked_steps += b->h_steps_left[d];
	}
	return pcg::sync_out(b);
}

int pcg_batch_prepare(pcg_batch* b)
{
	BATCH_CHECK(b);
	pcg::DeviceGuard g(b->device);
	int rc;
	if ((rc = pcg::refresh(b)))
		return rc;
	if (!b->use_graph)
		return PCG_OK;
	for (int rebuilds = 0; rebuilds < 2; rebuilds++)
		if (!b->exec[rebuilds] && (rc = pcg::capture(b, rebuilds)))
			return rc;
	return PCG_OK;
}

int pcg_batch_synchronize(pcg_batch* b)
{
	BATCH_CHECK(b);
	pcg::DeviceGuard g(b->device);
	return pcg::check_batch(b);
}

int pcg_batch_get_stream(pcg_batch* b, void** stream)
{
	BATCH_CHECK(b);
	if (!stream)
		return fail(PCG_ERR_INVALID, "null argument");
	*stream = b->stream;
	return PCG_OK;
}

int pcg_batch_set_graph(pcg_batch* b, int enable)
{
	BATCH_CHECK(b);
	b->use_graph = enable != 0;
	return PCG_OK;
}

int pcg_batch_autotune(pcg_batch* b)
{
	BATCH_CHECK(b);
	pcg::DeviceGuard g(b->device);
	int rc;
	if ((rc = pcg::sync_in(b)))
		return rc;
	rc = b->wsize == 4 ? pcg::autotune_t<float>(b) : pcg::autotune_t<double>(b);
	if (rc)
		return rc;
	return pcg::sync_out(b);
}

int pcg_batch_force_config(pcg_batch* b, int axis, int mapping, uint32_t rows)
{
	BATCH_CHECK(b);
	if (axis < 0 || axis > 2)
		return fail(PCG_ERR_INVALID, "axis must be 0, 1 or 2");
	if (mapping > 1 || (axis > 0 && mapping > 0))
		return fail(PCG_ERR_INVALID, "unknown mapping for this axis");
	b->forced[axis] = mapping >= 0;
	b->force[axis].mode = (uint32_t)std::max(mapping, 0);
	b->force[axis].rows = rows;
	b->built = false;
	return PCG_OK;
}

int pcg_batch_describe(pcg_batch* b, char* text, uint64_t cap, uint64_t* needed)
{
	BATCH_CHECK(b);
	const std::string s = pcg::describe(b);
	if (needed)
		*needed = s.size() + 1;
	if (text && cap)
	{
		const size_t n = std::min<size_t>(cap - 1, s.size());
		memcpy(text, s.data(), n);
		text[n] = 0;
	}
	return PCG_OK;
}

int pcg_batch_set_kernel_timing(pcg_batch* b, int enable)
{
	BATCH_CHECK(b);
	b->timing = enable != 0;
	return PCG_OK;
}

int pcg_batch_get_kernel_stats(pcg_batch* b, pcg_kernel_stat* stats, uint64_t cap, uint64_t* count)
{
	BATCH_CHECK(b);
	pcg::DeviceGuard g(b->device);
	pcg::batch_wait(b);
	pcg::collect(b);
	if (count)
		*count = pcg::K_COUNT;
	for (uint64_t k = 0; stats && k < cap && k < (uint64_t)pcg::K_COUNT; k++)
	{
		memset(&stats[k], 0, sizeof(pcg_kernel_stat));
		snprintf(stats[k].name, sizeof(stats[k].name), "%s", pcg::kernel_name((int)k));
		stats[k].launches = b->stats[k].launches;
		stats[k].total_ms = b->stats[k].total_ms;
		stats[k].algorithmic_bytes = b->stats[k].bytes;
	}
	return PCG_OK;
}

int pcg_batch_reset_kernel_stats(pcg_batch* b)
{
	BATCH_CHECK(b);
	pcg::DeviceGuard g(b->device);
	pcg::batch_wait(b);
	pcg::collect(b);
	for (auto& s : b->stats)
		s = pcg::KernelStat {};
	b->launches = 0;
	return PCG_OK;
}

int pcg_batch_get_launch_count(pcg_batch* b, uint64_t* launches)
{
	BATCH_CHECK(b);
	if (!launches)
		return fail(PCG_ERR_INVALID, "null argument");
	*launches = b->launches;
	return PCG_OK;
}

} // extern "C"
