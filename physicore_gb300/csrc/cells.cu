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
#include "pcg_internal.cuh"

namespace pcg {

namespace {

constexpr uint32_t kNoAgent = 0xffffffffu;

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
	void *num, *den, *fac, *rnum, *rden, *rfac;
	uint32_t* owner;
	uint32_t* counts;
	uint32_t* flags; // [0] conflict
	uint32_t* err;
	void* field;
	int internalized;
};

// cartesian_mesh::voxel_position (mesh.cpp:37-61); false when outside the grid.
__device__ __forceinline__ bool locate(const CellArgs& a, uint64_t i, uint64_t idx[3])
{
	idx[0] = idx[1] = idx[2] = 0;
	for (int d = 0; d < a.dims; d++)
	{
		const double q = (a.pos[i * a.dims + d] - a.bbmin[d]) / a.voxel[d];
		if (!(q >= 0.0) || q >= (double)a.n[d])
			return false;
		idx[d] = (uint64_t)q;
	}
	return true;
}

// compute_intermediates + clear_ballots (cell_solver.cpp:22-77)
template <typename T>
__global__ void cells_locate_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i == 0)
		a.flags[0] = 0;
	if (i >= a.A)
		return;
	uint64_t idx[3];
	if (!a.active[i])
	{
		a.vox[i] = kNoAgent;
		return;
	}
	if (!locate(a, i, idx))
	{
		atomicOr(a.err, DEV_ERR_AGENT_OUTSIDE);
		a.vox[i] = kNoAgent;
		return;
	}
	const uint32_t v = (uint32_t)(idx[0] + a.n[0] * (idx[1] + a.n[1] * idx[2]));
	a.vox[i] = v;
	a.foff[i] = (uint32_t)((idx[2] * a.n[1] + idx[1]) * a.pitch + idx[0] * a.S);
	a.owner[v] = kNoAgent;
	T* num = static_cast<T*>(a.num);
	T* den = static_cast<T*>(a.den);
	T* fac = static_cast<T*>(a.fac);
	T* rnum = static_cast<T*>(a.rnum);
	T* rden = static_cast<T*>(a.rden);
	T* rfac = static_cast<T*>(a.rfac);
	const double vol = a.vol[i];
	for (uint64_t s = 0; s < a.S; s++)
	{
		const uint64_t k = i * a.S + s;
		num[k] = (T)(a.sec[k] * a.sat[k] * a.dt * vol / a.Vv);
		den[k] = (T)((a.upt[k] + a.sec[k]) * a.dt * vol / a.Vv);
		fac[k] = (T)(a.net[k] * a.dt / a.Vv);
		rnum[k] = T(0);
		rden[k] = T(0);
		rfac[k] = T(0);
	}
}

// ballot (cell_solver.cpp:79-101 with a canonical winner)
__global__ void cells_ballot_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	const uint32_t key = i < a.A ? a.vox[i] : kNoAgent;
	const uint32_t group = __match_any_sync(0xffffffffu, key);
	if (key == kNoAgent)
		return;
	const int lane = threadIdx.x & 31;
	if (lane == __ffs(group) - 1)
	{
		// lanes of a warp hold consecutive agent indices, so the leader is the group minimum
		atomicMin(a.owner + key, (uint32_t)i);
		atomicAdd(a.counts + key, (uint32_t)__popc(group));
	}
}

// sums into the winner's row (cell_solver.cpp:102-127)
template <typename T>
__global__ void cells_reduce_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	const uint32_t key = i < a.A ? a.vox[i] : kNoAgent;
	bool conflict = false;
	if (key != kNoAgent)
	{
		const uint32_t w = a.owner[key];
		conflict = w != (uint32_t)i;
		const T* num = static_cast<const T*>(a.num);
		const T* den = static_cast<const T*>(a.den);
		const T* fac = static_cast<const T*>(a.fac);
		T* rnum = static_cast<T*>(a.rnum);
		T* rden = static_cast<T*>(a.rden);
		T* rfac = static_cast<T*>(a.rfac);
		for (uint64_t s = 0; s < a.S; s++)
		{
			const uint64_t k = i * a.S + s;
			const uint64_t kw = (uint64_t)w * a.S + s;
			atomicAdd(rnum + kw, num[k]);
			atomicAdd(rden + kw, conflict ? den[k] : den[k] + T(1));
			atomicAdd(rfac + kw, fac[k]);
		}
	}
	if (__any_sync(0xffffffffu, conflict) && (threadIdx.x & 31) == 0)
		atomicOr(a.flags, 1u);
}

constexpr int kSubBatch = 8; // substrates whose loads are issued together

// compute_result (cell_solver.cpp:187-227).  All loads of a batch of substrates are
// issued before any store, so an agent's independent memory accesses overlap.
template <typename T>
__global__ void cells_apply_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i >= a.A)
		return;
	const uint32_t key = a.vox[i];
	if (key == kNoAgent)
		return;
	const uint32_t off = a.foff[i];
	const bool fused = a.internalized && *(volatile uint32_t*)a.flags == 0;
	if (!fused && a.owner[key] != (uint32_t)i)
		return;
	T* __restrict__ D = static_cast<T*>(a.field) + off;
	const T* __restrict__ rn = static_cast<const T*>(a.rnum) + i * a.S;
	const T* __restrict__ rd = static_cast<const T*>(a.rden) + i * a.S;
	const T* __restrict__ rf = static_cast<const T*>(a.rfac) + i * a.S;
	double* __restrict__ I = a.internal + i * a.S;
	for (uint32_t s0 = 0; s0 < a.S; s0 += kSubBatch)
	{
		T dv[kSubBatch], n_[kSubBatch], d_[kSubBatch], f_[kSubBatch];
		double iv[kSubBatch];
#pragma unroll
		for (int q = 0; q < kSubBatch; q++)
			if (s0 + q < a.S)
			{
				dv[q] = D[s0 + q];
				n_[q] = rn[s0 + q];
				d_[q] = rd[s0 + q];
				f_[q] = rf[s0 + q];
				if (fused)
					iv[q] = I[s0 + q];
			}
#pragma unroll
		for (int q = 0; q < kSubBatch; q++)
			if (s0 + q < a.S)
			{
				const T next = (dv[q] + n_[q]) / d_[q] + f_[q];
				D[s0 + q] = next;
				if (fused)
					I[s0 + q] = iv[q] + a.Vv * ((double)dv[q] - (double)next);
			}
	}
}

// compute_internalized after a conflict (cell_solver.cpp:229-243)
template <typename T>
__global__ void cells_internalize_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i >= a.A)
		return;
	if (*(volatile uint32_t*)a.flags == 0)
		return;
	if (a.vox[i] == kNoAgent)
		return;
	const T* __restrict__ D = static_cast<const T*>(a.field) + a.foff[i];
	const T* __restrict__ nu = static_cast<const T*>(a.num) + i * a.S;
	const T* __restrict__ de = static_cast<const T*>(a.den) + i * a.S;
	const T* __restrict__ fa = static_cast<const T*>(a.fac) + i * a.S;
	double* __restrict__ I = a.internal + i * a.S;
	for (uint32_t s0 = 0; s0 < a.S; s0 += kSubBatch)
	{
		T dv[kSubBatch], n_[kSubBatch], d_[kSubBatch], f_[kSubBatch];
		double iv[kSubBatch];
#pragma unroll
		for (int q = 0; q < kSubBatch; q++)
			if (s0 + q < a.S)
			{
				dv[q] = D[s0 + q];
				n_[q] = nu[s0 + q];
				d_[q] = de[s0 + q];
				f_[q] = fa[s0 + q];
				iv[q] = I[s0 + q];
			}
#pragma unroll
		for (int q = 0; q < kSubBatch; q++)
			if (s0 + q < a.S)
				I[s0 + q] = iv[q] - a.Vv * ((double)n_[q] - (double)dv[q] * (double)d_[q] + (double)f_[q]);
	}
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
	*D = (T)((double)*D + a.internal[k] * a.frac[k] / a.Vv);
	a.internal[k] = 0.0;
}

CellArgs make_args(Context* c)
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
	a.flags = static_cast<uint32_t*>(c->flags.ptr);
	a.err = static_cast<uint32_t*>(c->err.ptr);
	a.field = c->field.ptr;
	a.internalized = c->compute_internalized ? 1 : 0;
	return a;
}

} // namespace

template <typename T>
static int run_cells(Context* c, bool recompute)
{
	if (c->A == 0)
		return PCG_OK;
	CellArgs a = make_args(c);
	const unsigned block = 256;
	const unsigned grid = (unsigned)((c->A + block - 1) / block);
	const double S = (double)c->S, A = (double)c->A, w = (double)sizeof(T);
	cudaEvent_t ev;
	if (recompute)
	{
		PCG_CUDA_TRY(cudaMemsetAsync(c->counts.ptr, 0, c->V * sizeof(uint32_t), c->stream));
		launch_begin(c, K_CELLS_LOCATE, A * (8.0 * c->dims + 1 + 5 * S * 8 + 8 + 6 * S * w + 4), &ev);
		cells_locate_kernel<T><<<grid, block, 0, c->stream>>>(a);
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
	// per active agent: voxel index, offset, reduced terms, density read+write
	launch_begin(c, K_CELLS_APPLY, A * (8 + 3 * S * w + 2 * S * w + (c->compute_internalized ? 16 * S : 0)), &ev);
	cells_apply_kernel<T><<<grid, block, 0, c->stream>>>(a);
	launch_end(c, K_CELLS_APPLY, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	if (c->compute_internalized)
	{
		// after a conflict: own terms, density read, internalized read+write
		launch_begin(c, K_CELLS_INTERNALIZE, A * (8 + 3 * S * w + S * w + 16 * S), &ev);
		cells_internalize_kernel<T><<<grid, block, 0, c->stream>>>(a);
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
	a.flags = b.flags;
	a.err = b.err;
	a.field = b.field;
	a.internalized = b.internalized;
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
	CellArgs a = make_args(c);
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
