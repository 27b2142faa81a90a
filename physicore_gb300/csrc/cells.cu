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
//  * locate: one thread per agent computes its voxel index in FP64 exactly as
//    cartesian_mesh::voxel_position does (mesh.cpp:37-61), so agent->voxel maps
//    and therefore the per-voxel counts are bit-exact with the reference.
//  * ballot: lanes holding the same voxel are grouped with __match_any_sync; the
//    group leader issues one atomicMin (the winner is the lowest agent index,
//    which canonicalises the reference's first-CAS-wins race) and one atomicAdd
//    of the group's population.
//  * reduce: each agent adds its terms into its winner's row with atomics (the
//    winner also adds the 1 of the denominator); any agent that is not its
//    voxel's winner raises the conflict flag, which stays on the device, so the
//    step never waits on the host (the Thrust backend copies it back every step,
//    thrust_solver/src/cell_solver.cpp:251-252).
//  * apply/internalize read the flag on the device and take the reference's
//    fused or two-pass branch.  A voxel's substrates are adjacent in the field, so
//    each agent touches one 32-byte sector of densities (S <= 8, FP32).
//  Internalized substrates are kept in FP64 in both builds.
#include "cells_device.cuh"

namespace pcg {

namespace {

using namespace cellsdev;

template <typename T>
__global__ void cells_locate_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i == 0)
		a.flags[0] = a.flags[1] = 0;
	if (i < a.A)
		agent_locate<T>(a, i);
}

__global__ void cells_ballot_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	const uint32_t key = i < a.A ? a.vox[i] : kNoAgent;
	// lanes of a warp hold consecutive agent indices, so a group's leader is its minimum
	warp_ballot(&a, i, key, key);
}

template <typename T>
__global__ void cells_reduce_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	const uint8_t role = i < a.A ? agent_reduce<T>(a, i) : kRoleNone;
	if (__any_sync(0xffffffffu, role == kRoleLoser) && (threadIdx.x & 31) == 0)
		atomicOr(a.flags, 1u);
	list_shared(a, i, role == kRoleWinner || role == kRoleLoser, 0);
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

// Over the list of agents in shared voxels (empty when there was no conflict).
template <typename T>
__global__ void cells_internalize_kernel(CellArgs a)
{
	const uint32_t count = __ldg(a.flags + 1);
	for (uint64_t j = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; j < count; j += (uint64_t)gridDim.x * blockDim.x)
		agent_internalize<T>(a, __ldg(a.shared + j));
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
	a.num = c->a_num.ptr;
	a.den = c->a_den.ptr;
	a.fac = c->a_fac.ptr;
	a.rnum = c->a_rnum.ptr;
	a.rden = c->a_rden.ptr;
	a.rfac = c->a_rfac.ptr;
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
	return a;
}

} // namespace cellsdev

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
	if (recompute)
	{
		PCG_CUDA_TRY(cudaMemsetAsync(c->counts.ptr, 0, c->V * sizeof(uint32_t), c->stream));
		// positions, activity, voxel index/offset, ballot slot, cleared sums; the terms
		// (rates, volume in; three FP32/FP64 rows out) only after new agent data
		a.terms = c->terms_dirty ? 1 : 0;
		launch_begin(c, K_CELLS_LOCATE,
					 A * (8.0 * c->dims + 1 + 8 + 4 + 3 * S * w + (a.terms ? 5 * S * 8 + 8 + 3 * S * w : 0)), &ev);
		cells_locate_kernel<T><<<grid, block, 0, c->stream>>>(a);
		c->terms_dirty = false;
		launch_end(c, K_CELLS_LOCATE, ev);
		PCG_CUDA_TRY(cudaGetLastError());
		launch_begin(c, K_CELLS_BALLOT, A * (4 + 8), &ev);
		cells_ballot_kernel<<<grid, block, 0, c->stream>>>(a);
		launch_end(c, K_CELLS_BALLOT, ev);
		PCG_CUDA_TRY(cudaGetLastError());
		launch_begin(c, K_CELLS_REDUCE, A * (8 + 6 * S * w), &ev);
		cells_reduce_kernel<T><<<grid, block, 0, c->stream>>>(a);
		launch_end(c, K_CELLS_REDUCE, ev);
		PCG_CUDA_TRY(cudaGetLastError());
	}
	// per agent: role, offset, summed (or own) terms, density read+write
	launch_begin(c, K_CELLS_APPLY, A * (5 + 3 * S * w + 2 * S * w + (c->compute_internalized ? 16 * S : 0)), &ev);
	cells_apply_kernel<T><<<grid, block, 0, c->stream>>>(a);
	launch_end(c, K_CELLS_APPLY, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	if (c->compute_internalized)
	{
		// the agents that share a voxel (a few percent at 1e6 agents in 320^3 voxels)
		// read their own terms and density and rewrite their internalized amounts:
		// not counted, only the list length is
		launch_begin(c, K_CELLS_INTERNALIZE, 4, &ev);
		cells_internalize_kernel<T><<<std::min<unsigned>(grid, 8 * std::max(c->sm_count, 1)), block, 0, c->stream>>>(a);
		launch_end(c, K_CELLS_INTERNALIZE, ev);
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
	const uint64_t V = b.n[0] * b.n[1] * b.n[2];
	const unsigned block = 256;
	const unsigned grid = (unsigned)((b.A + block - 1) / block);
	PCG_CUDA_TRY(cudaMemsetAsync(b.counts, 0, V * sizeof(uint32_t), stream));
	cells_locate_kernel<float><<<grid, block, 0, stream>>>(a);
	cells_ballot_kernel<<<grid, block, 0, stream>>>(a);
	cells_reduce_kernel<float><<<grid, block, 0, stream>>>(a);
	cells_apply_kernel<float><<<grid, block, 0, stream>>>(a);
	if (b.internalized)
		cells_internalize_kernel<float><<<grid, block, 0, stream>>>(a);
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
