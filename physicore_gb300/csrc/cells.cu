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
//    fused or two-pass branch.
//  Internalized substrates are kept in FP64 in both builds; the FP32 build
//  differences densities in FP64 before accumulating them.
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
	uint64_t pitch, plane;
	double Vv, dt;
	const double *pos, *sec, *sat, *upt, *net, *vol, *frac;
	const uint8_t* active;
	double* internal;
	uint32_t* foff;
	void *num, *den, *fac, *rnum, *rden, *rfac;
	uint32_t* owner;
	uint32_t* counts;
	uint32_t* flags; // [0] conflict
	uint32_t* err;
	void* field;
	int internalized;
};

// compute_intermediates + clear_ballots (cell_solver.cpp:22-77)
template <typename T>
__global__ void cells_locate_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i == 0)
		a.flags[0] = 0;
	if (i >= a.A)
		return;
	if (!a.active[i])
	{
		a.foff[i] = kNoAgent;
		return;
	}
	uint64_t idx[3] = { 0, 0, 0 };
	bool inside = true;
	for (int d = 0; d < a.dims; d++)
	{
		const double p = a.pos[i * a.dims + d];
		const double q = (p - a.bbmin[d]) / a.voxel[d];
		if (!(q >= 0.0) || q >= (double)a.n[d])
		{
			inside = false;
			break;
		}
		idx[d] = (uint64_t)q;
	}
	if (!inside)
	{
		atomicOr(a.err, DEV_ERR_AGENT_OUTSIDE);
		a.foff[i] = kNoAgent;
		return;
	}
	const uint32_t off = (uint32_t)((idx[2] * a.n[1] + idx[1]) * a.pitch + idx[0]);
	a.foff[i] = off;
	a.owner[off] = kNoAgent;
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
	const uint32_t key = i < a.A ? a.foff[i] : kNoAgent;
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
	const uint32_t key = i < a.A ? a.foff[i] : kNoAgent;
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

// compute_result (cell_solver.cpp:187-227)
template <typename T>
__global__ void cells_apply_kernel(CellArgs a)
{
	const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (i >= a.A)
		return;
	const uint32_t key = a.foff[i];
	if (key == kNoAgent)
		return;
	const bool conflict = *(volatile uint32_t*)a.flags != 0;
	const T* rnum = static_cast<const T*>(a.rnum);
	const T* rden = static_cast<const T*>(a.rden);
	const T* rfac = static_cast<const T*>(a.rfac);
	T* field = static_cast<T*>(a.field);
	if (a.internalized && !conflict)
	{
		for (uint64_t s = 0; s < a.S; s++)
		{
			const uint64_t k = i * a.S + s;
			T* D = field + s * a.plane + key;
			const T prev = *D;
			const T next = (prev + rnum[k]) / rden[k] + rfac[k];
			*D = next;
			a.internal[k] += a.Vv * ((double)prev - (double)next);
		}
		return;
	}
	if (a.owner[key] != (uint32_t)i)
		return;
	for (uint64_t s = 0; s < a.S; s++)
	{
		const uint64_t k = i * a.S + s;
		T* D = field + s * a.plane + key;
		*D = (*D + rnum[k]) / rden[k] + rfac[k];
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
	const uint32_t key = a.foff[i];
	if (key == kNoAgent)
		return;
	const T* num = static_cast<const T*>(a.num);
	const T* den = static_cast<const T*>(a.den);
	const T* fac = static_cast<const T*>(a.fac);
	const T* field = static_cast<const T*>(a.field);
	for (uint64_t s = 0; s < a.S; s++)
	{
		const uint64_t k = i * a.S + s;
		const double D = (double)field[s * a.plane + key];
		a.internal[k] -= a.Vv * ((double)num[k] - D * (double)den[k] + (double)fac[k]);
	}
}

// release_internal (cell_solver.cpp:274-289) for one agent
template <typename T>
__global__ void cells_release_kernel(CellArgs a, uint64_t agent)
{
	const uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
	if (s >= a.S)
		return;
	uint64_t idx[3] = { 0, 0, 0 };
	for (int d = 0; d < a.dims; d++)
	{
		const double q = (a.pos[agent * a.dims + d] - a.bbmin[d]) / a.voxel[d];
		if (!(q >= 0.0) || q >= (double)a.n[d])
		{
			atomicOr(a.err, DEV_ERR_AGENT_OUTSIDE);
			return;
		}
		idx[d] = (uint64_t)q;
	}
	const uint64_t off = (idx[2] * a.n[1] + idx[1]) * a.pitch + idx[0];
	T* field = static_cast<T*>(a.field);
	const uint64_t k = agent * a.S + s;
	const double add = a.internal[k] * a.frac[k] / a.Vv;
	field[s * a.plane + off] = (T)((double)field[s * a.plane + off] + add);
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
	a.plane = c->plane;
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
		PCG_CUDA_TRY(cudaMemsetAsync(c->counts.ptr, 0, c->plane * sizeof(uint32_t), c->stream));
		launch_begin(c, K_CELLS_LOCATE, A * (8.0 * c->dims + 1 + 5 * S * 8 + 4 + 6 * S * w + 4), &ev);
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
	launch_begin(c, K_CELLS_APPLY, A * (4 + 4 + 3 * S * w + 2 * S * w + (c->compute_internalized ? 16 * S : 0)), &ev);
	cells_apply_kernel<T><<<grid, block, 0, c->stream>>>(a);
	launch_end(c, K_CELLS_APPLY, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	if (c->compute_internalized)
	{
		launch_begin(c, K_CELLS_INTERNALIZE, A * 4, &ev);
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
