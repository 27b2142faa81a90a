// cells_device.cuh -- per-agent device code of the cell secretion/uptake step,
// shared by the single-domain kernels (cells.cu) and the batched ones (batch.cu).
//
// Arithmetic follows openmp_solver/src/cell_solver.cpp:
//   intermediates (51-77)   num = S*T*dt*Vc/Vv, den = (U+S)*dt*Vc/Vv, fac = N*dt/Vv
//   ballot        (79-129)  one winner per voxel collects sum(num), 1+sum(den), sum(fac)
//   result       (131-244)  D' = (D + sum num)/(1 + sum den) + sum fac by the winner;
//                           internalized: fused I += Vv (D - D') when no voxel holds two
//                           agents, otherwise I -= Vv (num - D' den + fac) per agent
//   release      (274-289)  D += I F / Vv, I = 0
#pragma once

#include "pcg_internal.cuh"

namespace pcg {
namespace cellsdev {

constexpr uint32_t kNoAgent = 0xffffffffu;
constexpr int kSubBatch = 8; // substrates whose loads are issued together

// Ballot role of an agent, recorded by agent_reduce whenever the ballot is rebuilt.
enum : uint8_t
{
	kRoleNone = 0,   // inactive or outside the grid
	kRoleAlone = 1,  // the only agent of its voxel
	kRoleWinner = 2, // winner of a voxel that holds several agents
	kRoleLoser = 3,  // any other agent of such a voxel (a ballot conflict)
};

struct CellArgs
{
	int dims;
	uint64_t A, S;
	uint64_t n[3];
	double bbmin[3];
	double voxel[3];
	uint64_t pitch;
	double Vv, dt;
	const double *pos, *sec, *sat, *upt, *net, *vol, *frac;
	const uint8_t* active;
	double* internal;
	uint32_t* vox;
	uint32_t* foff;
	// cell terms of agent i at num/den/fac + i * ts (S values each), the winner's
	// sums at rnum/rden/rfac + i * ts: a context keeps the three side by side in
	// one row (ts = term_stride(S)), caller-owned buffers as separate arrays (ts = S)
	void *num, *den, *fac, *rnum, *rden, *rfac;
	uint64_t ts;
	uint32_t* owner;
	uint32_t* counts;
	uint8_t* role;    // [A] ballot role
	uint32_t* shared; // [A] agents of voxels that hold several, flags[list_word] of them
	uint32_t* flags;  // [0] conflict; entries of `shared` in word list_word; grouped ballot: [2..4]
	uint32_t list_word; // 1 (batches: per-warp ballot) or 2 (grouped ballot: words 2, 3 = list, slots;
	                    // 4 = writers)
	uint32_t* err;
	void* field;
	int internalized;
	int vec;   // rows of S values start on 16-byte boundaries and S is a multiple of 16 / sizeof(T)
	int pairs; // internalized amounts stored as float pairs (FP32 contexts; see pair_add)
	int terms; // recompute the agent terms (their rates or volumes changed), not only positions
	// fast voxel location (locate): bbmin and 1/voxel as floats; fast == 0 when the
	// mesh's bounds or voxel edges are not exactly representable in FP32
	float mf[3], rf[3];
	int fast;
	// voxel-grouped ballot (cells.cu): rank of each agent in its voxel, and the
	// agents of shared voxels grouped by voxel (slot order)
	uint32_t* rank;   // [A]
	uint2* sorted;    // [A] (agent, voxel) pairs
	// a context's grouped ballot (null for caller-owned buffers): the agents that
	// write a voxel, flags[4] of them, in agent order (apply walks them instead of
	// every agent)
	uint32_t* writers;
};

// The fast-location constants of a mesh: float bounds and reciprocal voxel edges,
// usable when every bound and edge is an integer of at most 24 bits.
inline void set_fast_locate(CellArgs& a)
{
	a.fast = 1;
	for (int d = 0; d < a.dims; d++)
	{
		const double m = a.bbmin[d], h = a.voxel[d];
		if (!(fabs(m) <= 16777216.0) || !(h >= 1.0 && h <= 16777216.0) || (double)(float)m != m ||
			(double)(float)h != h || a.n[d] > (1u << 22))
			a.fast = 0;
		a.mf[d] = (float)m;
		a.rf[d] = (float)(1.0 / h);
	}
}

// Cell arguments of a context's own buffers (cells.cu).
CellArgs make_cell_args(const Context* c);

// Whether the rows of S values of `a` (field, terms, internalized) all start on
// 16-byte boundaries, for 16-byte accesses.
inline int rows_vectorizable(const CellArgs& a, size_t wsize)
{
	auto al = [](const void* p) { return p == nullptr || reinterpret_cast<uintptr_t>(p) % 16 == 0; };
	return a.S % (16 / wsize) == 0 && (a.pitch * wsize) % 16 == 0 && (a.ts * wsize) % 16 == 0 && al(a.field) &&
		   al(a.internal) && al(a.num) &&
		   al(a.den) && al(a.fac) && al(a.rnum) && al(a.rden) && al(a.rfac);
}

// cartesian_mesh::voxel_position (mesh.cpp:37-61): idx = trunc(q) with the FP64
// quotient q = (p - bbmin) / voxel, outside the grid when !(q >= 0) or q >= n;
// false when outside.  The result is exactly the FP64 expression's, but the
// division (a long sequence on this GPU's slow FP64 pipe) runs only near a voxel
// boundary: qf = (float(p) - float(bbmin)) * float(1/voxel) is within
// 2^-24 (3|q| + |p|/voxel) of q (one rounding each of p, the difference, the
// reciprocal and the product; bbmin and voxel are exact as floats), so when qf
// lies more than 2^-21 (|qf| + |p|/voxel) + 2^-40 from every integer, q lies
// strictly inside the same unit interval and trunc(q), and the bounds test, are
// decided by qf.  Otherwise (and for NaN or huge positions) the FP64 division
// decides.
__device__ __forceinline__ bool locate_exact_axis(const CellArgs& a, double p, int d, uint64_t& idx)
{
	const double q = (p - a.bbmin[d]) / a.voxel[d];
	if (!(q >= 0.0) || q >= (double)a.n[d])
		return false;
	idx = (uint64_t)q;
	return true;
}

__device__ __forceinline__ bool locate(const CellArgs& a, uint64_t i, uint64_t idx[3])
{
	idx[0] = idx[1] = idx[2] = 0;
	for (int d = 0; d < a.dims; d++)
	{
		const double p = a.pos[i * a.dims + d];
		if (a.fast)
		{
			const float pf = (float)p;
			const float qf = __fmul_rn(__fsub_rn(pf, a.mf[d]), a.rf[d]);
			const float fl = floorf(qf);
			const float tol = fmaf(fabsf(qf) + fabsf(pf) * a.rf[d], 4.76837158e-7f, 9.09494702e-13f); // 2^-21, 2^-40
			if (qf - fl > tol && (fl + 1.0f) - qf > tol)
			{
				if (fl < 0.0f || fl >= (float)a.n[d])
					return false;
				idx[d] = (uint64_t)fl;
				continue;
			}
		}
		if (!locate_exact_axis(a, p, d, idx[d]))
			return false;
	}
	return true;
}

// compute_intermediates + clear_ballots (cell_solver.cpp:22-77) for agent i < A.
// The terms depend on the agent's rates and volume only: a recompute after the
// agents moved keeps them (a.terms == 0), with the same values the reference
// recomputes.  With a.terms they are computed for inactive agents too, so that an
// agent activated later finds its terms.
template <typename T>
__device__ __forceinline__ void agent_terms(const CellArgs& a, uint64_t i)
{
	T* num = static_cast<T*>(a.num);
	T* den = static_cast<T*>(a.den);
	T* fac = static_cast<T*>(a.fac);
	{
		const double vol = a.vol[i];
		// FP32 build: the agent's dt Vc / Vv and dt / Vv once, products per
		// substrate; within a few FP64 ulps of the reference's left-to-right
		// quotients before the rounding to FP32, and without the divisions (double
		// precision runs at a small fraction of the single-precision rate on this
		// GPU).  FP64 build: the reference's expressions.
		const double fv = a.dt * vol / a.Vv, ft = a.dt / a.Vv;
		for (uint64_t s = 0; s < a.S; s++)
		{
			const uint64_t k = i * a.S + s, t = i * a.ts + s;
			if constexpr (sizeof(T) == 4)
			{
				num[t] = (T)(a.sec[k] * a.sat[k] * fv);
				den[t] = (T)((a.upt[k] + a.sec[k]) * fv);
				fac[t] = (T)(a.net[k] * ft);
			}
			else
			{
				num[t] = (T)(a.sec[k] * a.sat[k] * a.dt * vol / a.Vv);
				den[t] = (T)((a.upt[k] + a.sec[k]) * a.dt * vol / a.Vv);
				fac[t] = (T)(a.net[k] * a.dt / a.Vv);
			}
		}
	}
}

// The voxel of agent i < A (vox, foff), or kNoAgent when it is inactive or outside
// the grid (a device error then); returns it.
__device__ __forceinline__ uint32_t agent_place(const CellArgs& a, uint64_t i)
{
	uint64_t idx[3];
	if (!a.active[i])
	{
		a.vox[i] = kNoAgent;
		return kNoAgent;
	}
	if (!locate(a, i, idx))
	{
		atomicOr(a.err, DEV_ERR_AGENT_OUTSIDE);
		a.vox[i] = kNoAgent;
		return kNoAgent;
	}
	const uint32_t v = (uint32_t)(idx[0] + a.n[0] * (idx[1] + a.n[1] * idx[2]));
	a.vox[i] = v;
	a.foff[i] = (uint32_t)((idx[2] * a.n[1] + idx[1]) * a.pitch + idx[0] * a.S);
	return v;
}

template <typename T>
__device__ __forceinline__ void agent_locate(const CellArgs& a, uint64_t i)
{
	if (a.terms)
		agent_terms<T>(a, i);
	const uint32_t v = agent_place(a, i);
	if (v == kNoAgent)
		return;
	a.owner[v] = kNoAgent;
	T* rnum = static_cast<T*>(a.rnum);
	T* rden = static_cast<T*>(a.rden);
	T* rfac = static_cast<T*>(a.rfac);
	for (uint64_t s = 0; s < a.S; s++)
	{
		const uint64_t k = i * a.ts + s;
		rnum[k] = T(0);
		rden[k] = T(0);
		rfac[k] = T(0);
	}
}

// Ballot of one warp (cell_solver.cpp:79-101 with a canonical winner).  `key`
// must be unique per voxel across everything the warp holds (kNoAgent for none);
// the lanes of a warp hold ascending agent indices of one domain per group.
__device__ __forceinline__ void warp_ballot(const CellArgs* a, uint64_t i, uint32_t v, uint32_t key)
{
	const uint32_t group = __match_any_sync(0xffffffffu, key);
	if (key == kNoAgent)
		return;
	if ((threadIdx.x & 31) == __ffs(group) - 1)
	{
		atomicMin(a->owner + v, (uint32_t)i); // the leader holds the group's lowest index
		atomicAdd(a->counts + v, (uint32_t)__popc(group));
	}
}

// Sums into the winner's row (cell_solver.cpp:102-127) and records agent i's
// role, which it returns (kRoleLoser: a ballot conflict).  An agent alone in its
// voxel adds nothing: its sums would be its own terms (0 + x, exactly), which
// agent_apply reads in their place.
template <typename T>
__device__ __forceinline__ uint8_t agent_reduce(const CellArgs& a, uint64_t i)
{
	const uint32_t v = a.vox[i];
	if (v == kNoAgent)
	{
		a.role[i] = kRoleNone;
		return kRoleNone;
	}
	const uint32_t w = a.owner[v];
	const bool conflict = w != (uint32_t)i;
	if (!conflict && a.counts[v] == 1)
	{
		a.role[i] = kRoleAlone;
		return kRoleAlone;
	}
	const uint8_t role = conflict ? kRoleLoser : kRoleWinner;
	a.role[i] = role;
	const T* num = static_cast<const T*>(a.num);
	const T* den = static_cast<const T*>(a.den);
	const T* fac = static_cast<const T*>(a.fac);
	T* rnum = static_cast<T*>(a.rnum);
	T* rden = static_cast<T*>(a.rden);
	T* rfac = static_cast<T*>(a.rfac);
	for (uint64_t s = 0; s < a.S; s++)
	{
		const uint64_t k = i * a.ts + s;
		const uint64_t kw = (uint64_t)w * a.ts + s;
		atomicAdd(rnum + kw, num[k]);
		// the winner adds the 1 of the denominator (FP64 builds; FP32 rows hold the
		// bare sum of den, see fp32_update)
		atomicAdd(rden + kw, (conflict || sizeof(T) == 4) ? den[k] : den[k] + T(1));
		atomicAdd(rfac + kw, fac[k]);
	}
	return role;
}

// Appends agent i to the list of agents in shared voxels, one atomic per group of
// lanes with the same `key` (the lanes of one domain).  All lanes of the warp call it.
__device__ __forceinline__ void list_shared(const CellArgs& a, uint64_t i, bool shared, uint32_t key)
{
	const uint32_t group = __match_any_sync(0xffffffffu, shared ? key : 0xffffffffu);
	if (!shared)
		return;
	const uint32_t lane = threadIdx.x & 31, leader = __ffs(group) - 1;
	uint32_t base = 0;
	if (lane == leader)
		base = atomicAdd(a.flags + 1, (uint32_t)__popc(group));
	base = __shfl_sync(group, base, leader);
	a.shared[base + __popc(group & ((1u << lane) - 1))] = (uint32_t)i;
}

// ---- voxel-grouped ballot (single-domain contexts)
//
// The reference sums every agent's terms into its voxel's winner with atomics
// (cell_solver.cpp:79-129).  When tens of agents share a voxel those atomics
// serialise on the winner's row, so here the ballot groups the agents of shared
// voxels by voxel instead and sums each group with a segmented warp reduction:
//   place:     voxel of each agent; a count per voxel (one atomic per run of
//              lanes in the voxel) whose returned offset gives the agent's rank
//              in its voxel (rank 0, the agent whose atomic landed first, is the
//              winner, as the first compare-and-swap wins in the reference)
//   classify:  roles from count and rank; the agents of shared voxels are listed
//              in agent order (for the internalized pass), so are the agents that
//              write a voxel (for apply), and each winner reserves its voxel's
//              group of slots
//   group:     every agent of a shared voxel writes (index, voxel) into its
//              voxel's group
//   group sum: warps reduce consecutive slots by voxel; a group that lies within
//              one warp is stored once, a group split across warps adds its parts
//              to the winner's row (cleared by classify) with atomics

// Runs of equal keys among the lanes of a warp: the first lane of the caller's run
// and the first lane after it (32 at the end of the warp).  All lanes call it.
__device__ __forceinline__ void key_run(uint32_t key, uint32_t& first, uint32_t& end)
{
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
	const uint32_t heads = __ballot_sync(0xffffffffu, lane == 0 || prev != key);
	first = 31 - __clz(heads & (0xffffffffu >> (31 - lane)));
	const uint32_t later = heads & (0xfffffffeu << lane);
	end = later ? __ffs(later) - 1 : 32;
}

// Counts agents i0 + 32 k into voxels v[k] (k < K) and records their ranks in
// their voxels: one atomic per run of lanes with the same voxel (agents given in
// voxel order share one; in random order each lane has its own, which costs less
// than grouping the lanes by voxel); the K chunks' atomics are in flight together.
// All lanes of the warp call it (v[k] = kNoAgent for none).
template <int K>
__device__ __forceinline__ void count_rank(const CellArgs& a, uint64_t i0, const uint32_t (&v)[K])
{
	const uint32_t lane = threadIdx.x & 31;
	uint32_t first[K], end[K], base[K];
#pragma unroll
	for (int k = 0; k < K; k++)
		key_run(v[k], first[k], end[k]);
#pragma unroll
	for (int k = 0; k < K; k++)
		base[k] = v[k] != kNoAgent && lane == first[k] ? atomicAdd(a.counts + v[k], end[k] - first[k]) : 0u;
#pragma unroll
	for (int k = 0; k < K; k++)
	{
		const uint32_t b = __shfl_sync(0xffffffffu, base[k], first[k]);
		if (v[k] != kNoAgent)
			a.rank[i0 + 32 * k] = b + (lane - first[k]);
	}
}

// Change of an internalized amount.  The FP64 build evaluates the reference's
// expressions in FP64 in its order: fused Vv (D - D') (cell_solver.cpp:166-185),
// after a conflict -Vv (num - D' den + fac) (cell_solver.cpp:132-143).  The FP32
// build evaluates them in FP32 (the product inside one fma; *_inc): double-
// precision arithmetic runs at a small fraction of the single-precision rate on
// this GPU.
__device__ __forceinline__ double fused_delta(double Vv, double D, double Dn) { return Vv * (D - Dn); }
__device__ __forceinline__ double conflict_delta(double Vv, double n, double Dn, double d, double f)
{
	return -(Vv * (n - Dn * d + f));
}
__device__ __forceinline__ float fused_inc(double Vv, float D, float Dn) { return (float)Vv * (D - Dn); }
__device__ __forceinline__ float conflict_inc(double Vv, float n, float Dn, float d, float f)
{
	return -(float)Vv * (fmaf(-Dn, d, n) + f);
}

// FP32 contexts store each internalized amount as an unevaluated pair of floats
// hi + lo (hi first in memory, the same 8 bytes as a double; about 48 significant
// bits) and accumulate the FP32 increments with error-free transformations
// (Knuth's TwoSum), so the per-step update needs no FP64 instruction; the host
// converts to and from doubles at the API.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
	s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

__device__ __forceinline__ double pair_add(double stored, float x)
{
	const unsigned long long bits = (unsigned long long)__double_as_longlong(stored);
	const float hi = __uint_as_float((unsigned)bits), lo = __uint_as_float((unsigned)(bits >> 32));
	float s, e, h2, l2;
	two_sum(hi, x, s, e);
	two_sum(s, __fadd_rn(lo, e), h2, l2);
	return __longlong_as_double(
		(long long)(((unsigned long long)__float_as_uint(l2) << 32) | (unsigned long long)__float_as_uint(h2)));
}

__device__ __forceinline__ double pair_value(double stored)
{
	const unsigned long long bits = (unsigned long long)__double_as_longlong(stored);
	return (double)__uint_as_float((unsigned)bits) + (double)__uint_as_float((unsigned)(bits >> 32));
}

// Adds the increment x to a stored amount: FP64 build in FP64; FP32 build into a
// float pair, or (caller-owned FP64 amounts) into the double.
__device__ __forceinline__ double accumulate(double stored, double x, int) { return stored + x; }
__device__ __forceinline__ double accumulate(double stored, float x, int pairs)
{
	return pairs ? pair_add(stored, x) : stored + (double)x;
}

// Accesses to values s0 .. s0 + kSubBatch - 1 (those below S) of an agent's row.
// With `vec` they are 16-byte accesses: the rows of a warp's agents are scattered,
// so an access costs an L1 wavefront per lane whatever its width, and 16-byte ones
// need a quarter (FP32) or half (FP64) as many.
template <typename T>
__device__ __forceinline__ void row_load(const T* __restrict__ p, uint32_t s0, uint32_t S, bool vec, T (&v)[kSubBatch])
{
	constexpr int L = 16 / sizeof(T);
	if (vec)
	{
#pragma unroll
		for (int q = 0; q < kSubBatch; q += L)
			if (s0 + q < S)
			{
				union
				{
					uint4 u;
					T t[L];
				} x;
				x.u = *reinterpret_cast<const uint4*>(p + s0 + q);
#pragma unroll
				for (int r = 0; r < L; r++)
					v[q + r] = x.t[r];
			}
		return;
	}
#pragma unroll
	for (int q = 0; q < kSubBatch; q++)
		if (s0 + q < S)
			v[q] = p[s0 + q];
}

template <typename T>
__device__ __forceinline__ void row_store(T* __restrict__ p, uint32_t s0, uint32_t S, bool vec, const T (&v)[kSubBatch])
{
	constexpr int L = 16 / sizeof(T);
	if (vec)
	{
#pragma unroll
		for (int q = 0; q < kSubBatch; q += L)
			if (s0 + q < S)
			{
				union
				{
					uint4 u;
					T t[L];
				} x;
#pragma unroll
				for (int r = 0; r < L; r++)
					x.t[r] = v[q + r];
				*reinterpret_cast<uint4*>(p + s0 + q) = x.u;
			}
		return;
	}
#pragma unroll
	for (int q = 0; q < kSubBatch; q++)
		if (s0 + q < S)
			p[s0 + q] = v[q];
}

// The FP32 density update of a voxel from its sums num, den, fac (den without the
// reference's added 1): D' = D + ((num - D den) / (1 + den) + fac), the
// reference's D' = (D + num) / (1 + den) + fac rearranged.  Formed as 1 + den in
// FP32, the reference's denominator keeps only the leading bits of a small den
// (den ~ 1e-3: about 14 of 24), and the density an agent drives its voxel towards
// is about num / den, so that rounding would bias the voxel's value by up to
// ~1e-4 relative every step in the same direction.  Here den keeps its full
// precision and 1 + den only scales the (small) correction.
__device__ __forceinline__ float fp32_update(float D, float num, float den, float fac)
{
	return D + (fmaf(-D, den, num) / (1.0f + den) + fac);
}

// compute_result (cell_solver.cpp:188-244) for agent i.  All loads of a batch of
// substrates are issued before any store, so an agent's accesses overlap.
//
// The winner of a voxel writes its new density from the voxel's sums: for an
// agent alone in its voxel these are its own terms (num, den, fac; FP64 builds
// add the 1 of the denominator in T as the ballot does, FP32 builds use
// fp32_update).  Internalized amounts: when no voxel holds two
// agents, the reference's fused update I += Vv (D - D'); otherwise every agent's
// I -= Vv (num - D' den + fac) from the final density of its voxel
// (cell_solver.cpp:229-243).  An agent alone in its voxel has just written that
// final density itself, so it applies the update here, from the same values, and
// agent_internalize takes only the agents of shared voxels.
template <typename T, int SC = 0>
__device__ __forceinline__ void agent_apply(const CellArgs& a, uint64_t i)
{
	const uint8_t role = a.role[i];
	const uint32_t off = a.foff[i];
	if (role == kRoleNone || role == kRoleLoser)
		return;
	const bool alone = role == kRoleAlone;
	const bool track = alone && a.internalized;
	const bool fused = track && __ldg(a.flags) == 0;
	const bool vec = a.vec;
	const uint32_t S = SC ? (uint32_t)SC : (uint32_t)a.S; // SC: S fixed at compile time (1-8), else 0
	T* __restrict__ D = static_cast<T*>(a.field) + off;
	const T* __restrict__ rn = static_cast<const T*>(alone ? a.num : a.rnum) + i * a.ts;
	const T* __restrict__ rd = static_cast<const T*>(alone ? a.den : a.rden) + i * a.ts;
	const T* __restrict__ rf = static_cast<const T*>(alone ? a.fac : a.rfac) + i * a.ts;
	double* __restrict__ I = a.internal + i * S;
	for (uint32_t s0 = 0; s0 < S; s0 += kSubBatch)
	{
		T dv[kSubBatch], n_[kSubBatch], d_[kSubBatch], f_[kSubBatch], nx[kSubBatch];
		double iv[kSubBatch];
		row_load(D, s0, S, vec, dv);
		row_load(rn, s0, S, vec, n_);
		row_load(rd, s0, S, vec, d_);
		row_load(rf, s0, S, vec, f_);
		if (track)
			row_load(I, s0, S, vec, iv);
#pragma unroll
		for (int q = 0; q < kSubBatch; q++)
			if (s0 + q < S)
			{
				if constexpr (sizeof(T) == 4)
					nx[q] = fp32_update(dv[q], n_[q], d_[q], f_[q]);
				else
					nx[q] = (dv[q] + n_[q]) / (alone ? d_[q] + T(1) : d_[q]) + f_[q];
				if constexpr (sizeof(T) == 4)
				{
					if (fused)
						iv[q] = accumulate(iv[q], fused_inc(a.Vv, dv[q], nx[q]), a.pairs);
					else if (track)
						iv[q] = accumulate(iv[q], conflict_inc(a.Vv, n_[q], nx[q], d_[q], f_[q]), a.pairs);
				}
				else
				{
					if (fused)
						iv[q] += fused_delta(a.Vv, dv[q], nx[q]);
					else if (track)
						iv[q] += conflict_delta(a.Vv, n_[q], nx[q], d_[q], f_[q]);
				}
			}
		row_store(D, s0, S, vec, nx);
		if (track)
			row_store(I, s0, S, vec, iv);
	}
}

// compute_internalized after a conflict (cell_solver.cpp:132-143) for agent i of
// a voxel that holds several agents (an entry of the shared list).
template <typename T, int SC = 0>
__device__ __forceinline__ void agent_internalize(const CellArgs& a, uint64_t i)
{
	const bool vec = a.vec;
	const uint32_t S = SC ? (uint32_t)SC : (uint32_t)a.S;
	const T* __restrict__ D = static_cast<const T*>(a.field) + a.foff[i];
	const T* __restrict__ nu = static_cast<const T*>(a.num) + i * a.ts;
	const T* __restrict__ de = static_cast<const T*>(a.den) + i * a.ts;
	const T* __restrict__ fa = static_cast<const T*>(a.fac) + i * a.ts;
	double* __restrict__ I = a.internal + i * S;
	for (uint32_t s0 = 0; s0 < S; s0 += kSubBatch)
	{
		T dv[kSubBatch], n_[kSubBatch], d_[kSubBatch], f_[kSubBatch];
		double iv[kSubBatch];
		row_load(D, s0, S, vec, dv);
		row_load(nu, s0, S, vec, n_);
		row_load(de, s0, S, vec, d_);
		row_load(fa, s0, S, vec, f_);
		row_load(I, s0, S, vec, iv);
#pragma unroll
		for (int q = 0; q < kSubBatch; q++)
			if (s0 + q < S)
			{
				if constexpr (sizeof(T) == 4)
					iv[q] = accumulate(iv[q], conflict_inc(a.Vv, n_[q], dv[q], d_[q], f_[q]), a.pairs);
				else
					iv[q] += conflict_delta(a.Vv, n_[q], dv[q], d_[q], f_[q]);
			}
		row_store(I, s0, S, vec, iv);
	}
}

} // namespace cellsdev
} // namespace pcg
