// cells.cu -- agent secretion/uptake with voxel ballots.
//
// Arithmetic follows openmp_solver/src/cell_solver.cpp:
//   intermediates (51-77)   num = S*T*dt*Vc/Vv, den = (U+S)*dt*Vc/Vv, fac = N*dt/Vv
//   ballot        (79-129)  one winner per voxel collects sum(num), 1+sum(den), sum(fac)
//   result       (131-244)  D' = (D + sum num)/(1 + sum den) + sum fac by the winner;
//                           internalized: fused I += Vv (D - D') when no voxel holds two
//                           agents, otherwise I -= Vv (num - D' den + fac) per agent
//   release      (274-289)  D += I F / Vv, I = 0
//
// GB300 design:
//  * place: one thread per agent computes its voxel index exactly as
//    cartesian_mesh::voxel_position does (mesh.cpp:37-61; locate in
//    cells_device.cuh: an FP32 estimate decides unless it lies within its error
//    bound of a voxel boundary, where the FP64 division decides), so the
//    agent->voxel maps and the per-voxel counts are bit-exact with the reference;
//    a run of lanes in one voxel counts with one atomic, whose returned offset
//    ranks the agents of the voxel.
//  * ballot: rank 0 wins the voxel (the reference's first compare-and-swap wins,
//    cell_solver.cpp:79-101); the agents of shared voxels are grouped by voxel and
//    each group is summed by a segmented warp reduction instead of every agent
//    adding its terms to the winner's row with contended atomics
//    (cell_solver.cpp:102-127); the conflict flag stays on the device, so the step
//    never waits on the host (the Thrust backend copies it back every step,
//    thrust_solver/src/cell_solver.cpp:251-252).
//  * apply (over the agents that write a voxel) and internalize (over the agents
//    of shared voxels) read the flag on the device and take the reference's
//    fused or two-pass branch.  A voxel's substrates are adjacent in the field, so
//    each agent touches one 32-byte sector of densities (S <= 8, FP32).
//  Batches keep the per-warp ballot with atomics (batch.cu).
#include "cells_device.cuh"

namespace pcg {

namespace {

using namespace cellsdev;

// place: terms (after new agent data), voxel, count and rank; the step's words
// (conflict flag, list length, reserved group slots) start at zero.  One agent
// per thread: two per thread (both chunks' loads and atomics in flight together)
// measured slower on the dense workload, 78 -> 107 us.
template <typename T>
__global__ void cells_place_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i == 0)
	{
		a.flags[0] = a.flags[1] = a.flags[2] = a.flags[3] = 0;
		if (a.writers)
			a.flags[4] = 0;
	}
	uint32_t v[1] = { kNoAgent };
	if (i < a.A)
	{
		if (a.terms)
			agent_terms<T>(a, i);
		v[0] = agent_place(a, i);
	}
	count_rank<1>(a, i, v);
}

constexpr unsigned kClassifyBlock = 1024;
constexpr unsigned kClassifyChunks = 4; // 32-agent chunks per warp

// classify: roles from count and rank (cell_solver.cpp:102-127: every agent but
// the winner of a shared voxel is a conflict); the agents of shared voxels listed
// in agent order (flags[2]); each winner reserves its voxel's group of slots
// (owner[v] = first slot, flags[3] counts slots) and clears its reduced row; with
// a writer list, the agents that write a voxel (alone or winner) listed in agent
// order (flags[4]).  A warp takes kClassifyChunks consecutive chunks of 32 agents
// (their loads in flight together).  A block scans its counts and reserves its
// ranges with one 64-bit atomic on the adjacent, 8-byte aligned words flags[2..3]
// (list entries low, slots high; neither total reaches 2^32, so no carry crosses)
// and one on flags[4]: same-address atomics that return a value serialise, so
// there is one per 4096 agents and word.
template <typename T>
__global__ void __launch_bounds__(kClassifyBlock, 2) cells_classify_kernel(CellArgs a)
{
	constexpr int K = kClassifyChunks;
	__shared__ uint32_t part[3][kClassifyBlock / 32];
	__shared__ uint32_t base[3];
	const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
	const uint64_t i0 = ((uint64_t)blockIdx.x * nw + warp) * (K * 32) + lane;
	uint32_t v[K], cnt[K];
	uint8_t role[K];
#pragma unroll
	for (int k = 0; k < K; k++)
	{
		const uint64_t i = i0 + k * 32;
		v[k] = i < a.A ? a.vox[i] : kNoAgent;
		cnt[k] = v[k] != kNoAgent ? a.rank[i] : 0u; // the rank, for now
	}
	// an agent of rank > 0 shares its voxel: only rank 0 needs the count (a
	// scattered read that the block's scans would wait for)
#pragma unroll
	for (int k = 0; k < K; k++)
	{
		const bool first = v[k] != kNoAgent && cnt[k] == 0;
		role[k] = v[k] == kNoAgent ? kRoleNone : (first ? kRoleWinner : kRoleLoser);
		cnt[k] = first ? a.counts[v[k]] : 0u;
	}
	bool loser = false;
	uint32_t bsh[K], bwr[K], seg_inc[K], tsh = 0, twr = 0, tseg = 0;
	const uint32_t below = (1u << lane) - 1u;
#pragma unroll
	for (int k = 0; k < K; k++)
	{
		const uint64_t i = i0 + k * 32;
		if (role[k] == kRoleWinner && cnt[k] == 1)
			role[k] = kRoleAlone;
		if (i < a.A)
			a.role[i] = role[k];
		loser |= role[k] == kRoleLoser;
		bsh[k] = __ballot_sync(0xffffffffu, role[k] == kRoleWinner || role[k] == kRoleLoser);
		bwr[k] = __ballot_sync(0xffffffffu, a.writers && (role[k] == kRoleAlone || role[k] == kRoleWinner));
		// slots before this lane's in the warp's agent order (chunk-major)
		uint32_t x = role[k] == kRoleWinner ? cnt[k] : 0u;
		for (uint32_t o = 1; o < 32; o <<= 1)
		{
			const uint32_t t = __shfl_up_sync(0xffffffffu, x, o);
			if (lane >= o)
				x += t;
		}
		seg_inc[k] = tseg + x;
		tseg += __shfl_sync(0xffffffffu, x, 31);
		tsh += __popc(bsh[k]);
		twr += __popc(bwr[k]);
	}
	if (__any_sync(0xffffffffu, loser) && lane == 0)
		atomicOr(a.flags, 1u);
	if (lane == 0)
		part[0][warp] = tsh, part[1][warp] = tseg, part[2][warp] = twr;
	__syncthreads();
	if (warp == 0)
	{
		uint32_t p[3];
#pragma unroll
		for (int q = 0; q < 3; q++)
			p[q] = lane < nw ? part[q][lane] : 0u;
		for (uint32_t o = 1; o < 32; o <<= 1)
#pragma unroll
			for (int q = 0; q < 3; q++)
			{
				const uint32_t t = __shfl_up_sync(0xffffffffu, p[q], o);
				if (lane >= o)
					p[q] += t;
			}
		if (lane == 31)
		{
			unsigned long long old = 0ull;
			if (p[0] | p[1])
				old = atomicAdd(reinterpret_cast<unsigned long long*>(a.flags + 2),
								((unsigned long long)p[1] << 32) | (unsigned long long)p[0]);
			base[0] = (uint32_t)old;
			base[1] = (uint32_t)(old >> 32);
			base[2] = p[2] ? atomicAdd(a.flags + 4, p[2]) : 0u;
		}
#pragma unroll
		for (int q = 0; q < 3; q++)
		{
			const uint32_t e = __shfl_up_sync(0xffffffffu, p[q], 1);
			if (lane < nw)
				part[q][lane] = lane == 0 ? 0u : e;
		}
	}
	__syncthreads();
	uint32_t osh = base[0] + part[0][warp], owr = base[2] + part[2][warp];
	const uint32_t oseg = base[1] + part[1][warp];
#pragma unroll
	for (int k = 0; k < K; k++)
	{
		const uint64_t i = i0 + k * 32;
		if ((bsh[k] >> lane) & 1u)
			a.shared[osh + __popc(bsh[k] & below)] = (uint32_t)i;
		if ((bwr[k] >> lane) & 1u)
			a.writers[owr + __popc(bwr[k] & below)] = (uint32_t)i;
		osh += __popc(bsh[k]);
		owr += __popc(bwr[k]);
		if (role[k] == kRoleWinner)
		{
			a.owner[v[k]] = oseg + seg_inc[k] - cnt[k];
			T* rn = static_cast<T*>(a.rnum) + i * a.ts;
			T* rd = static_cast<T*>(a.rden) + i * a.ts;
			T* rf = static_cast<T*>(a.rfac) + i * a.ts;
			for (uint64_t s = 0; s < a.S; s++)
				rn[s] = rd[s] = rf[s] = T(0);
		}
	}
}

// group: every agent of a shared voxel (role from classify) writes (its index,
// its voxel) into its voxel's group of slots.  One thread per agent: with many
// agents per voxel nearly all of them write, and the loads of one agent (role,
// voxel, rank, then its voxel's first slot) form a chain that only more threads in
// flight hide.
__global__ void cells_group_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i >= a.A)
		return;
	const uint8_t role = a.role[i];
	if (role != kRoleWinner && role != kRoleLoser)
		return;
	const uint32_t v = a.vox[i];
	a.sorted[(uint64_t)__ldg(a.owner + v) + a.rank[i]] = make_uint2((uint32_t)i, v);
}

// group sum: a warp takes 32 consecutive slots and sums each voxel's terms with a
// segmented scan (lanes of one voxel are consecutive); the last lane of each
// voxel's run writes the winner's row: sum num, sum den (plus 1 in FP64 builds),
// sum fac -- stored when the run is the voxel's whole group, else added with
// atomics (the part holding the group's first slot adds the 1).  SC is S when
// the launch fixes it at compile time (1-8: the per-substrate guards fold away),
// else 0.
template <typename T, int SC>
__global__ void cells_group_sum_kernel(CellArgs a)
{
	const uint32_t count = __ldg(a.flags + a.list_word);
	const uint32_t lane = threadIdx.x & 31;
	const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
	const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
	const uint32_t S = SC ? (uint32_t)SC : (uint32_t)a.S;
	const bool vec = a.vec;
	T* rnum = static_cast<T*>(a.rnum);
	T* rden = static_cast<T*>(a.rden);
	T* rfac = static_cast<T*>(a.rfac);
	for (uint64_t j0 = gw * 32; j0 < count; j0 += nwarps * 32)
	{
		const uint64_t j = j0 + lane;
		uint32_t v = kNoAgent;
		const T *pn = nullptr, *pd = nullptr, *pf = nullptr;
		if (j < count)
		{
			// the agent's three rows lie side by side in a context's term rows
			const uint2 iv = __ldg(a.sorted + j);
			v = iv.y;
			pn = static_cast<const T*>(a.num) + (uint64_t)iv.x * a.ts;
			pd = static_cast<const T*>(a.den) + (uint64_t)iv.x * a.ts;
			pf = static_cast<const T*>(a.fac) + (uint64_t)iv.x * a.ts;
		}
		uint32_t first, end;
		key_run(v, first, end);
		const uint32_t last = end - 1;
		const bool writer = v != kNoAgent && lane == last;
		uint32_t w = 0;
		bool head = false, whole = false;
		if (writer)
		{
			const uint32_t seg0 = __ldg(a.owner + v), cnt = __ldg(a.counts + v);
			w = __ldg(&a.sorted[seg0].x);
			head = j0 + first == seg0;
			whole = head && j0 + last == (uint64_t)seg0 + cnt - 1;
		}
		uint32_t kup[5];
#pragma unroll
		for (int k = 0; k < 5; k++)
			kup[k] = __shfl_up_sync(0xffffffffu, v, 1u << k);
		for (uint32_t s0 = 0; s0 < S; s0 += kSubBatch)
		{
			T n_[kSubBatch], d_[kSubBatch], f_[kSubBatch];
#pragma unroll
			for (int q = 0; q < kSubBatch; q++)
				n_[q] = d_[q] = f_[q] = T(0);
			if (v != kNoAgent)
			{
				row_load(pn, s0, S, vec, n_);
				row_load(pd, s0, S, vec, d_);
				row_load(pf, s0, S, vec, f_);
			}
#pragma unroll
			for (int k = 0; k < 5; k++)
			{
				const uint32_t o = 1u << k;
				const bool take = lane >= o && kup[k] == v;
#pragma unroll
				for (int q = 0; q < kSubBatch; q++)
					if (s0 + q < S) // uniform across the warp
					{
						const T tn = __shfl_up_sync(0xffffffffu, n_[q], o);
						const T td = __shfl_up_sync(0xffffffffu, d_[q], o);
						const T tf = __shfl_up_sync(0xffffffffu, f_[q], o);
						if (take)
							n_[q] += tn, d_[q] += td, f_[q] += tf;
					}
			}
			if (writer)
			{
				if (head && sizeof(T) == 8) // FP64 rows hold 1 + sum den; FP32 rows the bare sum (fp32_update)
#pragma unroll
					for (int q = 0; q < kSubBatch; q++)
						d_[q] += T(1);
				const uint64_t r = (uint64_t)w * a.ts;
				if (whole)
				{
					row_store(rnum + r, s0, S, vec, n_);
					row_store(rden + r, s0, S, vec, d_);
					row_store(rfac + r, s0, S, vec, f_);
				}
				else
#pragma unroll
					for (int q = 0; q < kSubBatch; q++)
						if (s0 + q < S)
						{
							atomicAdd(rnum + r + s0 + q, n_[q]);
							atomicAdd(rden + r + s0 + q, d_[q]);
							atomicAdd(rfac + r + s0 + q, f_[q]);
						}
			}
		}
	}
}

// FP32: registers capped for 3 blocks of 256 per SM (a latency-bound gather:
// more loads in flight; the FP64 build would spill)
template <typename T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) cells_apply_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i < a.A)
		agent_apply<T>(a, i);
}

// Over the agents that write a voxel (alone or winner; flags[4] of them, listed
// by classify) when they are fewer than half the agents, else over every agent
// (agent_apply returns at once for the others): with many agents per voxel most
// agents only lose their ballot, and a thread per agent would mostly wait on its
// role byte.  Grid-stride, so the grid need not match the device-side count.
// SC: S fixed at compile time (1-8), else 0.
template <typename T, int SC>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 1) cells_apply_writers_kernel(CellArgs a)
{
	const uint32_t count = __ldg(a.flags + 4);
	const bool list = 2ull * count < a.A;
	const uint64_t n = list ? count : a.A;
	for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < n; j += (uint64_t)gridDim.x * blockDim.x)
		agent_apply<T, SC>(a, list ? __ldg(a.writers + j) : j);
}

// Over the list of agents in shared voxels (empty when there was no conflict).
template <typename T, int SC>
__global__ void cells_internalize_kernel(CellArgs a)
{
	const uint32_t count = __ldg(a.flags + a.list_word);
	for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < count; j += (uint64_t)gridDim.x * blockDim.x)
		agent_internalize<T, SC>(a, __ldg(a.shared + j));
}

// Launches KERNEL<T, S> for S = 1..8, KERNEL<T, 0> otherwise.
#define PCG_LAUNCH_BY_S(KERNEL, T, S, GRID, BLOCK, STREAM, ARGS)                                                       \
	switch (S)                                                                                                         \
	{                                                                                                                  \
	case 1: KERNEL<T, 1><<<GRID, BLOCK, 0, STREAM>>>(ARGS); break;                                                   \
	case 2: KERNEL<T, 2><<<GRID, BLOCK, 0, STREAM>>>(ARGS); break;                                                   \
	case 3: KERNEL<T, 3><<<GRID, BLOCK, 0, STREAM>>>(ARGS); break;                                                   \
	case 4: KERNEL<T, 4><<<GRID, BLOCK, 0, STREAM>>>(ARGS); break;                                                   \
	case 5: KERNEL<T, 5><<<GRID, BLOCK, 0, STREAM>>>(ARGS); break;                                                   \
	case 6: KERNEL<T, 6><<<GRID, BLOCK, 0, STREAM>>>(ARGS); break;                                                   \
	case 7: KERNEL<T, 7><<<GRID, BLOCK, 0, STREAM>>>(ARGS); break;                                                   \
	case 8: KERNEL<T, 8><<<GRID, BLOCK, 0, STREAM>>>(ARGS); break;                                                   \
	default: KERNEL<T, 0><<<GRID, BLOCK, 0, STREAM>>>(ARGS);                                                         \
	}

// release_internal (cell_solver.cpp:274-289) for one agent
template <typename T>
__global__ void cells_release_kernel(CellArgs a, uint64_t agent)
{
	const uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (s >= a.S)
		return;
	uint64_t idx[3];
	if (!locate(a, agent, idx))
	{
		atomicOr(a.err, DEV_ERR_AGENT_OUTSIDE);
		return;
	}
	T* D = static_cast<T*>(a.field) + (idx[2] * a.n[1] + idx[1]) * a.pitch + idx[0] * a.S + s;
	const uint64_t k = agent * a.S + s;
	const double I = a.pairs ? pair_value(a.internal[k]) : a.internal[k];
	*D = (T)((double)*D + I * a.frac[k] / a.Vv);
	a.internal[k] = 0.0; // zero bits: a zero pair too
}

} // namespace

namespace cellsdev {

CellArgs make_cell_args(const Context* c)
{
	CellArgs a {};
	a.dims = c->dims;
	a.A = c->A;
	a.S = c->S;
	for (int d = 0; d < 3; d++)
	{
		a.n[d] = c->n[d];
		a.bbmin[d] = (double)c->bbmin[d];
		a.voxel[d] = (double)c->voxel[d];
	}
	a.pitch = c->pitch;
	a.Vv = (double)(c->voxel[0] * c->voxel[1] * c->voxel[2]);
	a.dt = c->dt;
	a.pos = static_cast<const double*>(c->a_pos.ptr);
	a.sec = static_cast<const double*>(c->a_sec.ptr);
	a.sat = static_cast<const double*>(c->a_sat.ptr);
	a.upt = static_cast<const double*>(c->a_upt.ptr);
	a.net = static_cast<const double*>(c->a_net.ptr);
	a.vol = static_cast<const double*>(c->a_vol.ptr);
	a.frac = static_cast<const double*>(c->a_frac.ptr);
	a.active = static_cast<const uint8_t*>(c->a_active.ptr);
	a.internal = static_cast<double*>(c->a_internal.ptr);
	a.vox = static_cast<uint32_t*>(c->a_vox.ptr);
	a.foff = static_cast<uint32_t*>(c->a_foff.ptr);
	// num, den and fac side by side in each agent's row
	const size_t rb = c->S * c->wsize;
	a.ts = c->term_stride;
	a.num = c->a_terms.ptr;
	a.den = static_cast<char*>(c->a_terms.ptr) + rb;
	a.fac = static_cast<char*>(c->a_terms.ptr) + 2 * rb;
	a.rnum = c->a_reduced.ptr;
	a.rden = static_cast<char*>(c->a_reduced.ptr) + rb;
	a.rfac = static_cast<char*>(c->a_reduced.ptr) + 2 * rb;
	a.owner = static_cast<uint32_t*>(c->owner.ptr);
	a.counts = static_cast<uint32_t*>(c->counts.ptr);
	a.role = static_cast<uint8_t*>(c->a_role.ptr);
	a.shared = static_cast<uint32_t*>(c->a_shared.ptr);
	a.flags = static_cast<uint32_t*>(c->flags.ptr);
	a.err = static_cast<uint32_t*>(c->err.ptr);
	a.field = c->field.ptr;
	a.internalized = c->compute_internalized ? 1 : 0;
	a.vec = rows_vectorizable(a, c->wsize);
	a.terms = 1;
	a.pairs = c->wsize == 4 ? 1 : 0; // FP32 contexts store internalized amounts as float pairs
	a.rank = static_cast<uint32_t*>(c->a_rank.ptr);
	a.sorted = static_cast<uint2*>(c->a_sorted.ptr);
	a.writers = static_cast<uint32_t*>(c->a_writers.ptr);
	a.list_word = 2; // the grouped ballot (a batch sets 1 for its per-warp ballot)
	set_fast_locate(a);
	return a;
}

} // namespace cellsdev

// The voxel-grouped ballot (cells_device.cuh) on `stream`; launch bookkeeping
// through `c` when given.
template <typename T>
static int run_ballot(Context* c, const CellArgs& a, cudaStream_t stream, int sm_count)
{
	const unsigned block = 256;
	const unsigned grid = (unsigned)((a.A + block - 1) / block);
	const uint64_t per_block = (uint64_t)kClassifyBlock * kClassifyChunks;
	const unsigned cgrid = (unsigned)((a.A + per_block - 1) / per_block);
	// the list of shared-voxel agents is only known on the device: grid-stride
	const unsigned lgrid = std::min<unsigned>(grid, 16 * std::max(sm_count, 1));
	const double S = (double)a.S, A = (double)a.A, w = (double)sizeof(T);
	cudaEvent_t ev = nullptr;
	if (c)
		launch_begin(c, K_CELLS_LOCATE,
					 A * (8.0 * a.dims + 1 + 4 + 4 + 4 + 4) + (a.terms ? A * (5 * S * 8 + 8 + 3 * S * w) : 0), &ev);
	cells_place_kernel<T><<<grid, block, 0, stream>>>(a);
	if (c)
		launch_end(c, K_CELLS_LOCATE, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	if (c)
		launch_begin(c, K_CELLS_BALLOT, A * (4 + 4 + 4 + 1), &ev);
	cells_classify_kernel<T><<<cgrid, kClassifyBlock, 0, stream>>>(a);
	if (c && c->timing && c->h_words) // list lengths for the per-agent byte counts
	{
		PCG_CUDA_TRY(
			cudaMemcpyAsync(c->h_words + 2, a.flags + a.list_word, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
		PCG_CUDA_TRY(cudaMemcpyAsync(c->h_words + 3, a.flags + 4, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream));
	}
	// shared-voxel agents: list entry, winner's row cleared; writers: list entry
	if (c)
		launch_end(c, K_CELLS_BALLOT, ev, 4.0 + 3 * S * w, 4.0);
	PCG_CUDA_TRY(cudaGetLastError());
	// per agent its role; per shared-voxel agent its voxel, rank and voxel's first
	// slot, and the pair written
	if (c)
		launch_begin(c, K_CELLS_GROUP, A, &ev);
	cells_group_kernel<<<grid, block, 0, stream>>>(a);
	if (c)
		launch_end(c, K_CELLS_GROUP, ev, 20.0);
	PCG_CUDA_TRY(cudaGetLastError());
	// per slot: the pair and the agent's three rows (one gathered term row in a
	// context)
	if (c)
		launch_begin(c, K_CELLS_REDUCE, 0.0, &ev);
	switch (a.S)
	{
#define PCG_GROUP_SUM(SV)                                                                                              \
	case SV:                                                                                                           \
		cells_group_sum_kernel<T, SV><<<lgrid, block, 0, stream>>>(a);                                                 \
		break;
		PCG_GROUP_SUM(1)
		PCG_GROUP_SUM(2)
		PCG_GROUP_SUM(3)
		PCG_GROUP_SUM(4)
		PCG_GROUP_SUM(5)
		PCG_GROUP_SUM(6)
		PCG_GROUP_SUM(7)
		PCG_GROUP_SUM(8)
#undef PCG_GROUP_SUM
	default:
		cells_group_sum_kernel<T, 0><<<lgrid, block, 0, stream>>>(a);
	}
	if (c)
		launch_end(c, K_CELLS_REDUCE, ev, 8.0 + 3 * S * w);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

template <typename T>
static int run_cells(Context* c, bool recompute)
{
	if (c->A == 0)
		return PCG_OK;
	CellArgs a = make_cell_args(c);
	const unsigned block = 256;
	const unsigned grid = (unsigned)((c->A + block - 1) / block);
	const double S = (double)c->S, A = (double)c->A, w = (double)sizeof(T);
	cudaEvent_t ev;
	// the cached roles and lists must come from this kind of ballot (a batch keeps
	// its own list and counts)
	if (c->ballot_kind != 1)
		recompute = true;
	if (recompute)
	{
		PCG_CUDA_TRY(cudaMemsetAsync(c->counts.ptr, 0, c->V * sizeof(uint32_t), c->stream));
		// the terms (rates, volume in; three rows out) only after new agent data
		a.terms = c->terms_dirty ? 1 : 0;
		if (c->timing && !c->h_words && !(c->h_words = pinned_words_get()))
			return fail(PCG_ERR_NOMEM, "pinned host memory for the device words");
		const int rc = run_ballot<T>(c, a, c->stream, c->sm_count);
		if (rc)
			return rc;
		c->terms_dirty = false;
		c->ballot_kind = 1;
	}
	// per writer: list entry, role, offset, summed (or own) terms, density read and
	// write, internalized amounts read and written
	launch_begin(c, K_CELLS_APPLY, 0.0, &ev);
	const unsigned agrid = std::min<unsigned>(grid, 24 * std::max(c->sm_count, 1));
	PCG_LAUNCH_BY_S(cells_apply_writers_kernel, T, c->S, agrid, block, c->stream, a);
	launch_end(c, K_CELLS_APPLY, ev, 0.0, 9 + 3 * S * w + 2 * S * w + (c->compute_internalized ? 16 * S : 0));
	PCG_CUDA_TRY(cudaGetLastError());
	if (c->compute_internalized)
	{
		// the agents that share a voxel (a few percent at 1e6 agents in 320^3 voxels):
		// list entry, offset, density, own terms, internalized read and write each
		launch_begin(c, K_CELLS_INTERNALIZE, 0.0, &ev);
		const unsigned igrid = std::min<unsigned>(grid, 24 * std::max(c->sm_count, 1));
		PCG_LAUNCH_BY_S(cells_internalize_kernel, T, c->S, igrid, block, c->stream, a);
		launch_end(c, K_CELLS_INTERNALIZE, ev, 8.0 + 4 * S * w + 16 * S);
		PCG_CUDA_TRY(cudaGetLastError());
	}
	return PCG_OK;
}

int launch_cells(Context* c, bool recompute)
{
	return c->wsize == 4 ? run_cells<float>(c, recompute) : run_cells<double>(c, recompute);
}

// The same kernels over caller-owned buffers: the counts are cleared here, the
// conflict flag, ballot slots and reduced terms by the locate kernel.
int launch_cells_fp32_buffers(const CellStepBuffers& b, cudaStream_t stream)
{
	if (b.A == 0)
		return PCG_OK;
	CellArgs a {};
	a.dims = b.dims;
	a.A = b.A;
	a.S = b.S;
	for (int d = 0; d < 3; d++)
	{
		a.n[d] = b.n[d];
		a.bbmin[d] = (double)b.bbmin[d];
		a.voxel[d] = (double)b.voxel[d];
	}
	a.pitch = b.pitch;
	a.Vv = (double)(b.voxel[0] * b.voxel[1] * b.voxel[2]);
	a.dt = b.dt;
	a.pos = b.pos;
	a.sec = b.sec;
	a.sat = b.sat;
	a.upt = b.upt;
	a.net = b.net;
	a.vol = b.vol;
	a.frac = nullptr;
	a.active = b.active;
	a.internal = b.internal;
	a.vox = b.vox;
	a.foff = b.foff;
	a.num = b.num;
	a.den = b.den;
	a.fac = b.fac;
	a.rnum = b.rnum;
	a.rden = b.rden;
	a.rfac = b.rfac;
	a.ts = b.S; // separate arrays
	a.owner = b.owner;
	a.counts = b.counts;
	a.role = b.role;
	a.shared = b.shared;
	a.flags = b.flags;
	a.err = b.err;
	a.field = b.field;
	a.internalized = b.internalized;
	a.vec = rows_vectorizable(a, sizeof(float));
	a.terms = 1;
	a.pairs = 0; // the caller's FP64 amounts
	a.rank = b.rank;
	a.sorted = b.sorted;
	a.list_word = 2;
	set_fast_locate(a);
	const uint64_t V = b.n[0] * b.n[1] * b.n[2];
	const unsigned block = 256;
	const unsigned grid = (unsigned)((b.A + block - 1) / block);
	int sm_count = 0, dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev) !=
												   cudaSuccess)
		sm_count = 0;
	PCG_CUDA_TRY(cudaMemsetAsync(b.counts, 0, V * sizeof(uint32_t), stream));
	int rc = run_ballot<float>(nullptr, a, stream, sm_count);
	if (rc)
		return rc;
	cells_apply_kernel<float><<<grid, block, 0, stream>>>(a);
	if (b.internalized)
		cells_internalize_kernel<float, 0><<<grid, block, 0, stream>>>(a);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

template <typename T>
static int run_release(Context* c, uint64_t agent)
{
	CellArgs a = make_cell_args(c);
	cudaEvent_t ev;
	launch_begin(c, K_CELLS_RELEASE, (double)(c->S * 32), &ev);
	cells_release_kernel<T><<<(unsigned)((c->S + 63) / 64), 64, 0, c->stream>>>(a, agent);
	launch_end(c, K_CELLS_RELEASE, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

int launch_release(Context* c, uint64_t agent)
{
	return c->wsize == 4 ? run_release<float>(c, agent) : run_release<double>(c, agent);
}

} // namespace pcg
