// field_ops.cu -- Dirichlet, bulk source/sink, mass and layout kernels.
//
// Dirichlet faces and interior (openmp_solver/src/dirichlet_solver.cpp:22-93) and
// bulk (openmp_solver/src/bulk_solver.cpp:12-49): per-item bodies live in
// field_device.cuh; one launch covers all six faces, a second the interior list.
#include "field_device.cuh"

namespace pcg {

namespace {

template <typename T>
__global__ void dirichlet_faces_kernel(FaceArgs a)
{
	for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < a.total * a.S;
		 idx += (uint64_t)gridDim.x * blockDim.x)
		fielddev::face_item<T>(a, idx);
}

template <typename T>
__global__ void dirichlet_interior_kernel(T* field, const uint64_t* offsets, const T* values, const uint8_t* conds,
										  uint64_t K, uint64_t S)
{
	for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < K * S;
		 idx += (uint64_t)gridDim.x * blockDim.x)
	{
		if (conds[idx])
			field[offsets[idx / S] + idx % S] = values[idx];
	}
}

// A warp per row.
template <typename T, bool PER_VOXEL>
__global__ void bulk_kernel(T* field, const T* supply, const T* uptake, const T* target, uint64_t row_len,
							uint64_t pitch, uint64_t rows, uint32_t S, T dt)
{
	const int lane = threadIdx.x & 31;
	const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
	const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
	for (uint64_t r = warp; r < rows; r += nwarps)
		fielddev::bulk_row<T, PER_VOXEL>(field, supply, uptake, target, row_len, pitch, r, S, dt, lane);
}

// FP64 mass per substrate: a warp per row, one substrate at a time.
template <typename T>
__global__ void mass_kernel(const T* field, double* out, uint64_t nx, uint64_t pitch, uint64_t rows, uint32_t S)
{
	const int lane = threadIdx.x & 31;
	const uint64_t warp = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
	const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
	for (uint32_t s = 0; s < S; s++)
	{
		double acc = 0.0;
		for (uint64_t r = warp; r < rows; r += nwarps)
		{
			const T* row = field + r * pitch + s;
			for (uint64_t x = lane; x < nx; x += 32)
				acc += (double)row[x * S];
		}
		for (int o = 16; o > 0; o >>= 1)
			acc += __shfl_xor_sync(0xffffffffu, acc, o);
		if (lane == 0)
			atomicAdd(out + s, acc);
	}
}

// One small block after a checked step's sweeps: per substrate, the totals the
// sweeps added before (tot[0, S)) and after (tot[S, 2S)), the worst relative
// residual of after * factor = before, and the totals cleared for the next step.
// out = [before S | after S | worst S | factor S].
__global__ void mass_check_finish_kernel(double* tot, uint32_t S, double* out)
{
	for (uint32_t s = threadIdx.x; s < S; s += blockDim.x)
	{
		const double b = tot[s], a = tot[S + s];
		out[s] = b;
		out[S + s] = a;
		const double res = fabs(a * out[3 * S + s] - b) / fmax(fabs(b), 1e-300);
		out[2 * S + s] = fmax(out[2 * S + s], res);
		tot[s] = 0.0;
		tot[S + s] = 0.0;
	}
}

template <typename T>
__global__ void fill_kernel(T* field, const T* init, uint64_t row_len, uint64_t pitch, uint64_t rows, uint32_t S)
{
	const uint64_t total = rows * pitch;
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
		 i += (uint64_t)gridDim.x * blockDim.x)
	{
		const uint64_t k = i % pitch;
		field[i] = k < row_len ? init[k % S] : T(0);
	}
}

// Device field <-> dense host-order buffer of element type OUT/IN.
// Interleaved host layout [v][s]: element order equals the device row order, so
// consecutive threads read consecutive device values.
template <typename T, typename OUT>
__global__ void pack_interleaved_kernel(const T* field, OUT* dst, uint64_t nx, uint64_t pitch, uint64_t rows,
										uint64_t S)
{
	const uint64_t row_len = nx * S, total = row_len * rows;
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
		 i += (uint64_t)gridDim.x * blockDim.x)
		dst[i] = (OUT)field[(i / row_len) * pitch + i % row_len];
}

// Planar host layout [s][v]: a thread per voxel reads the voxel's S adjacent
// values once and writes one value into each substrate's plane (coalesced across
// the warp for every s).
template <typename T, typename OUT>
__global__ void pack_planar_kernel(const T* field, OUT* dst, uint64_t nx, uint64_t pitch, uint64_t rows, uint32_t S)
{
	const uint64_t V = nx * rows;
	for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x)
	{
		const T* src = field + (v / nx) * pitch + (v % nx) * S;
		for (uint32_t s = 0; s < S; s++)
			dst[s * V + v] = (OUT)src[s];
	}
}

template <typename T, typename IN>
__global__ void unpack_interleaved_kernel(T* field, const IN* src, uint64_t nx, uint64_t pitch, uint64_t rows,
										  uint64_t S)
{
	const uint64_t row_len = nx * S, total = row_len * rows;
	for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < total;
		 i += (uint64_t)gridDim.x * blockDim.x)
		field[(i / row_len) * pitch + i % row_len] = (T)src[i];
}

template <typename T, typename IN>
__global__ void unpack_planar_kernel(T* field, const IN* src, uint64_t nx, uint64_t pitch, uint64_t rows, uint32_t S)
{
	const uint64_t V = nx * rows;
	for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x)
	{
		T* out = field + (v / nx) * pitch + (v % nx) * S;
		for (uint32_t s = 0; s < S; s++)
			out[s] = (T)src[s * V + v];
	}
}

unsigned grid_for(const Context* c, uint64_t work, unsigned block)
{
	uint64_t g = (work + block - 1) / block;
	const uint64_t cap = (uint64_t)(c->sm_count > 0 ? c->sm_count : 152) * 16;
	if (g > cap)
		g = cap;
	return (unsigned)(g ? g : 1);
}

} // namespace

template <typename T>
static int run_dirichlet(Context* c, bool faces_done)
{
	const FaceArgs a = make_face_args(c);
	if (a.face_mask && !faces_done)
	{
		cudaEvent_t ev;
		launch_begin(c, K_DIRICHLET_FACES, (double)(a.total * c->S * sizeof(T)), &ev);
		dirichlet_faces_kernel<T><<<grid_for(c, a.total * c->S, 256), 256, 0, c->stream>>>(a);
		launch_end(c, K_DIRICHLET_FACES, ev);
		PCG_CUDA_TRY(cudaGetLastError());
	}
	if (c->K)
	{
		cudaEvent_t ev;
		launch_begin(c, K_DIRICHLET_INTERIOR, (double)(c->K * (8 + c->S * (2 * sizeof(T) + 1))), &ev);
		dirichlet_interior_kernel<T><<<grid_for(c, c->K * c->S, 256), 256, 0, c->stream>>>(
			static_cast<T*>(c->field.ptr), static_cast<const uint64_t*>(c->dir_offsets.ptr),
			static_cast<const T*>(c->dir_values.ptr), static_cast<const uint8_t*>(c->dir_conds.ptr), c->K, c->S);
		launch_end(c, K_DIRICHLET_INTERIOR, ev);
		PCG_CUDA_TRY(cudaGetLastError());
	}
	return PCG_OK;
}

int launch_dirichlet(Context* c, bool faces_done)
{
	return c->wsize == 4 ? run_dirichlet<float>(c, faces_done) : run_dirichlet<double>(c, faces_done);
}

template <typename T>
static int run_bulk(Context* c)
{
	if (c->bulk_mode == PCG_BULK_NONE)
		return PCG_OK;
	const bool pv = c->bulk_mode == PCG_BULK_PER_VOXEL;
	const unsigned grid = grid_for(c, c->rows * 32, 256);
	cudaEvent_t ev;
	const double bytes = (double)(c->V * c->S * sizeof(T)) * (pv ? 5.0 : 2.0);
	launch_begin(c, K_BULK, bytes, &ev);
	const T* sp = static_cast<const T*>(c->bulk[0].ptr);
	const T* up = static_cast<const T*>(c->bulk[1].ptr);
	const T* tp = static_cast<const T*>(c->bulk[2].ptr);
	if (pv)
		bulk_kernel<T, true><<<grid, 256, 0, c->stream>>>(static_cast<T*>(c->field.ptr), sp, up, tp, c->row_len,
														  c->pitch, c->rows, (uint32_t)c->S, (T)c->dt);
	else
		bulk_kernel<T, false><<<grid, 256, 0, c->stream>>>(static_cast<T*>(c->field.ptr), sp, up, tp, c->row_len,
														   c->pitch, c->rows, (uint32_t)c->S, (T)c->dt);
	launch_end(c, K_BULK, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

int launch_bulk(Context* c) { return c->wsize == 4 ? run_bulk<float>(c) : run_bulk<double>(c); }

template <typename T>
static int run_mass(Context* c, double* out)
{
	PCG_CUDA_TRY(cudaMemsetAsync(out, 0, c->S * sizeof(double), c->stream));
	cudaEvent_t ev;
	launch_begin(c, K_MASS, (double)(c->V * c->S * sizeof(T)), &ev);
	mass_kernel<T><<<grid_for(c, c->rows * 32, 256), 256, 0, c->stream>>>(static_cast<const T*>(c->field.ptr), out,
																		   c->n[0], c->pitch, c->rows,
																		   (uint32_t)c->S);
	launch_end(c, K_MASS, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

int launch_mass(Context* c, double* out) { return c->wsize == 4 ? run_mass<float>(c, out) : run_mass<double>(c, out); }

int launch_mass_check_finish(Context* c)
{
	cudaEvent_t ev;
	launch_begin(c, K_MASS_CHECK, (double)(c->S * 6 * sizeof(double)), &ev);
	mass_check_finish_kernel<<<1, 64, 0, c->stream>>>(static_cast<double*>(c->mc_tot.ptr), (uint32_t)c->S,
													  static_cast<double*>(c->mc_out.ptr));
	launch_end(c, K_MASS_CHECK, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

template <typename T>
static int run_fill(Context* c)
{
	cudaEvent_t ev;
	launch_begin(c, K_LAYOUT, (double)(c->rows * c->pitch * sizeof(T)), &ev);
	fill_kernel<T><<<grid_for(c, c->rows * c->pitch, 256), 256, 0, c->stream>>>(
		static_cast<T*>(c->field.ptr), static_cast<const T*>(c->mass.ptr), c->row_len, c->pitch, c->rows,
		(uint32_t)c->S);
	launch_end(c, K_LAYOUT, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

int launch_fill_initial(Context* c) { return c->wsize == 4 ? run_fill<float>(c) : run_fill<double>(c); }

template <typename T, typename H>
static int run_pack(Context* c, void* dst, int layout)
{
	const uint64_t total = c->V * c->S;
	cudaEvent_t ev;
	launch_begin(c, K_LAYOUT, (double)(total * (sizeof(T) + sizeof(H))), &ev);
	if (layout == PCG_LAYOUT_INTERLEAVED)
		pack_interleaved_kernel<T, H><<<grid_for(c, total, 256), 256, 0, c->stream>>>(
			static_cast<const T*>(c->field.ptr), static_cast<H*>(dst), c->n[0], c->pitch, c->rows, c->S);
	else
		pack_planar_kernel<T, H><<<grid_for(c, c->V, 256), 256, 0, c->stream>>>(
			static_cast<const T*>(c->field.ptr), static_cast<H*>(dst), c->n[0], c->pitch, c->rows, (uint32_t)c->S);
	launch_end(c, K_LAYOUT, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

template <typename T, typename H>
static int run_unpack(Context* c, const void* src, int layout)
{
	const uint64_t total = c->V * c->S;
	cudaEvent_t ev;
	launch_begin(c, K_LAYOUT, (double)(total * (sizeof(T) + sizeof(H))), &ev);
	if (layout == PCG_LAYOUT_INTERLEAVED)
		unpack_interleaved_kernel<T, H><<<grid_for(c, total, 256), 256, 0, c->stream>>>(
			static_cast<T*>(c->field.ptr), static_cast<const H*>(src), c->n[0], c->pitch, c->rows, c->S);
	else
		unpack_planar_kernel<T, H><<<grid_for(c, c->V, 256), 256, 0, c->stream>>>(
			static_cast<T*>(c->field.ptr), static_cast<const H*>(src), c->n[0], c->pitch, c->rows, (uint32_t)c->S);
	launch_end(c, K_LAYOUT, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

int launch_to_host_layout(Context* c, void* dst, int layout, int dtype)
{
	if (c->wsize == 4)
		return dtype == PCG_DTYPE_F32 ? run_pack<float, float>(c, dst, layout) : run_pack<float, double>(c, dst, layout);
	return dtype == PCG_DTYPE_F32 ? run_pack<double, float>(c, dst, layout) : run_pack<double, double>(c, dst, layout);
}

int launch_from_host_layout(Context* c, const void* src, int layout, int dtype)
{
	if (c->wsize == 4)
		return dtype == PCG_DTYPE_F32 ? run_unpack<float, float>(c, src, layout)
									  : run_unpack<float, double>(c, src, layout);
	return dtype == PCG_DTYPE_F32 ? run_unpack<double, float>(c, src, layout)
								  : run_unpack<double, double>(c, src, layout);
}

} // namespace pcg
