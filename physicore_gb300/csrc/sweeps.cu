// sweeps.cu -- ADI/LOD Thomas sweeps along x, y and z on sm_103a.
//
// Arithmetic per line follows the reference (openmp_solver/src/diffusion_solver.cpp:
// 116-202 for x, 390-794 for y/z; the coefficients of diffusion_solver.cpp:29-86):
//   forward   d_i  = d_i + e_{i-1} d_{i-1}            i = 1..n-1
//             d_{n-1} = d_{n-1} b'_{n-1}
//   backward  d_i  = (d_i + c d_{i+1}) b'_i            i = n-2..0
//
// GB300 mapping (our own design):
//  * y/z sweeps: a tile is 32 consecutive x positions of all n points of the
//    lines of one (substrate, outer) pair.  Its n rows of 128 B (FP32) are pulled
//    into shared memory by TMA bulk copies (cp.async.bulk) completing on an
//    mbarrier; lane t then solves line t out of shared memory (column t of an
//    [n][32] tile: bank-conflict free), and the tile goes back by bulk copies.
//  * x sweep: lines run along the contiguous axis, so a tile is 32 whole rows;
//    each row is one bulk copy into a shared-memory row whose pitch is 16 B
//    modulo 128 B, and lane r walks row r with 16-byte vector accesses (8 lanes
//    of a quarter-warp hit 8 distinct 16-byte bank groups).
//  * The per-substrate coefficient tables (b', e padded to 16 B) travel with the
//    tile in the same bulk transaction; every lane reads them as broadcasts.
//  * Every wait is bounded; a timeout sets a device error bit and the CTA exits
//    after its own copies have drained.
#include "pcg_internal.cuh"

namespace pcg {

namespace {

template <typename T>
struct Vec16;
template <>
struct Vec16<float>
{
	using type = float4;
	static constexpr int N = 4;
};
template <>
struct Vec16<double>
{
	using type = double2;
	static constexpr int N = 2;
};

template <typename T>
__device__ __forceinline__ T vget(const typename Vec16<T>::type& v, int u);
template <>
__device__ __forceinline__ float vget<float>(const float4& v, int u)
{
	return u == 0 ? v.x : u == 1 ? v.y : u == 2 ? v.z : v.w;
}
template <>
__device__ __forceinline__ double vget<double>(const double2& v, int u)
{
	return u == 0 ? v.x : v.y;
}
template <typename T>
__device__ __forceinline__ void vset(typename Vec16<T>::type& v, int u, T x);
template <>
__device__ __forceinline__ void vset<float>(float4& v, int u, float x)
{
	if (u == 0)
		v.x = x;
	else if (u == 1)
		v.y = x;
	else if (u == 2)
		v.z = x;
	else
		v.w = x;
}
template <>
__device__ __forceinline__ void vset<double>(double2& v, int u, double x)
{
	if (u == 0)
		v.x = x;
	else
		v.y = x;
}

__host__ __device__ inline uint64_t round_up(uint64_t v, uint64_t m) { return (v + m - 1) / m * m; }

__device__ __forceinline__ float fmadd(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmadd(double a, double b, double c) { return __fma_rn(a, b, c); }

// -------------------------------------------------------------------- y / z

template <typename T>
__global__ void __launch_bounds__(kSweepLanes) sweep_yz_kernel(SweepYZArgs a)
{
	extern __shared__ __align__(128) unsigned char smem[];
	uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
	const uint64_t npad = a.coef_pitch / 2;
	T* sB = reinterpret_cast<T*>(smem + 16);
	T* sE = sB + npad;
	T* tile = sB + a.coef_pitch;

	const uint64_t t = blockIdx.x;
	if (t >= a.tiles)
		return;
	const uint64_t xb = t % a.xblocks;
	const uint64_t rest = t / a.xblocks;
	const uint64_t o = rest % a.outer_count;
	const uint64_t s = rest / a.outer_count;
	const uint64_t x0 = xb * kSweepLanes;
	const uint64_t valid = a.nx - x0 < (uint64_t)kSweepLanes ? a.nx - x0 : (uint64_t)kSweepLanes;
	const uint32_t row_bytes = (uint32_t)round_up(valid * sizeof(T), 16);
	const uint32_t coef_bytes = (uint32_t)(a.coef_pitch * sizeof(T));
	const uint32_t n = (uint32_t)a.n;

	T* gbase = static_cast<T*>(a.field) + s * a.plane + o * a.outer_stride + x0;
	const T* gcoef = static_cast<const T*>(a.coef) + s * a.coef_pitch;
	const int lane = threadIdx.x;

	if (lane == 0)
	{
		dev::mbar_init(bar, 1);
		dev::fence_mbar_init();
	}
	__syncwarp();
	if (lane == 0)
		dev::mbar_arrive_expect_tx(bar, coef_bytes + n * row_bytes);
	__syncwarp();
	if (lane == 0)
		dev::bulk_g2s(sB, gcoef, coef_bytes, bar);
	for (uint32_t j = lane; j < n; j += kSweepLanes)
		dev::bulk_g2s(tile + (uint64_t)j * kSweepLanes, gbase + j * a.line_stride, row_bytes, bar);

	if (!dev::mbar_wait(bar, 0))
	{
		if (lane == 0)
			atomicOr(a.err, DEV_ERR_WAIT_TIMEOUT);
		return;
	}

	if ((uint64_t)lane < valid)
	{
		const T c = static_cast<const T*>(a.coef_c)[s];
		T* col = tile + lane;
		T d = col[0];
#pragma unroll 8
		for (uint32_t j = 1; j < n; j++)
		{
			d = fmadd(sE[j], d, col[(uint64_t)j * kSweepLanes]);
			col[(uint64_t)j * kSweepLanes] = d;
		}
		d = d * sB[n - 1];
		col[(uint64_t)(n - 1) * kSweepLanes] = d;
#pragma unroll 8
		for (int j = (int)n - 2; j >= 0; j--)
		{
			d = fmadd(c, d, col[(uint64_t)j * kSweepLanes]) * sB[j];
			col[(uint64_t)j * kSweepLanes] = d;
		}
	}
	dev::fence_proxy_async_smem();
	__syncwarp();
	for (uint32_t j = lane; j < n; j += kSweepLanes)
		dev::bulk_s2g(gbase + j * a.line_stride, tile + (uint64_t)j * kSweepLanes, row_bytes);
	dev::bulk_commit();
	dev::bulk_wait_all();
}

// -------------------------------------------------------------------- x

template <typename T>
__global__ void __launch_bounds__(kSweepXRows) sweep_x_kernel(SweepXArgs a)
{
	using V = typename Vec16<T>::type;
	constexpr int VN = Vec16<T>::N;
	extern __shared__ __align__(128) unsigned char smem[];
	uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
	const uint64_t npad = a.coef_pitch / 2;
	T* sB = reinterpret_cast<T*>(smem + 16);
	T* sE = sB + npad;
	T* rows = sB + a.coef_pitch;

	const uint64_t t = blockIdx.x;
	if (t >= a.tiles)
		return;
	const uint64_t rb = t % a.rblocks;
	const uint64_t s = t / a.rblocks;
	const uint64_t r0 = rb * kSweepXRows;
	const uint64_t nrows = a.rows - r0 < (uint64_t)kSweepXRows ? a.rows - r0 : (uint64_t)kSweepXRows;
	const uint32_t n = (uint32_t)a.n;
	const uint32_t row_bytes = (uint32_t)(npad * sizeof(T));
	const uint32_t coef_bytes = (uint32_t)(a.coef_pitch * sizeof(T));
	const uint64_t plane = a.rows * a.pitch;

	T* gbase = static_cast<T*>(a.field) + s * plane + r0 * a.pitch;
	const T* gcoef = static_cast<const T*>(a.coef) + s * a.coef_pitch;
	const int lane = threadIdx.x;

	if (lane == 0)
	{
		dev::mbar_init(bar, 1);
		dev::fence_mbar_init();
	}
	__syncwarp();
	if (lane == 0)
		dev::mbar_arrive_expect_tx(bar, coef_bytes + (uint32_t)nrows * row_bytes);
	__syncwarp();
	if (lane == 0)
		dev::bulk_g2s(sB, gcoef, coef_bytes, bar);
	if ((uint64_t)lane < nrows)
		dev::bulk_g2s(rows + lane * a.smem_pitch, gbase + lane * a.pitch, row_bytes, bar);

	if (!dev::mbar_wait(bar, 0))
	{
		if (lane == 0)
			atomicOr(a.err, DEV_ERR_WAIT_TIMEOUT);
		return;
	}

	if ((uint64_t)lane < nrows)
	{
		const T c = static_cast<const T*>(a.coef_c)[s];
		V* row = reinterpret_cast<V*>(rows + lane * a.smem_pitch);
		const V* vE = reinterpret_cast<const V*>(sE);
		const V* vB = reinterpret_cast<const V*>(sB);
		const uint32_t nv = (n + VN - 1) / VN;
		T d = T(0);
		// forward elimination; E[0] = 0 makes the first point pass through unchanged
		for (uint32_t k = 0; k < nv; k++)
		{
			V v = row[k];
			const V e = vE[k];
#pragma unroll
			for (int u = 0; u < VN; u++)
			{
				if (k * VN + u < n)
				{
					d = fmadd(vget<T>(e, u), d, vget<T>(v, u));
					vset<T>(v, u, d);
				}
			}
			row[k] = v;
		}
		// back substitution
		for (int k = (int)nv - 1; k >= 0; k--)
		{
			V v = row[k];
			const V b = vB[k];
#pragma unroll
			for (int u = VN - 1; u >= 0; u--)
			{
				const uint32_t i = (uint32_t)k * VN + u;
				if (i == n - 1)
				{
					d = vget<T>(v, u) * vget<T>(b, u);
					vset<T>(v, u, d);
				}
				else if (i < n - 1)
				{
					d = fmadd(c, d, vget<T>(v, u)) * vget<T>(b, u);
					vset<T>(v, u, d);
				}
			}
			row[k] = v;
		}
	}
	dev::fence_proxy_async_smem();
	__syncwarp();
	if ((uint64_t)lane < nrows)
		dev::bulk_s2g(gbase + lane * a.pitch, rows + lane * a.smem_pitch, row_bytes);
	dev::bulk_commit();
	dev::bulk_wait_all();
}

} // namespace

// -------------------------------------------------------------------- host side

uint64_t sweep_x_smem_pitch(const Context* c)
{
	const uint64_t chunk = 16 / c->wsize; // elements per 16-byte chunk
	uint64_t chunks = round_up(c->n[0], chunk) / chunk;
	chunks += (1 + 8 - chunks % 8) % 8; // chunks per row == 1 (mod 8): conflict-free 16-byte lanes
	return chunks * chunk;
}

uint64_t sweep_x_smem_bytes(const Context* c)
{
	return 16 + c->coef_pitch[0] * c->wsize + (uint64_t)kSweepXRows * sweep_x_smem_pitch(c) * c->wsize;
}

uint64_t sweep_yz_smem_bytes(const Context* c, int axis)
{
	return 16 + c->coef_pitch[axis] * c->wsize + c->n[axis] * (uint64_t)kSweepLanes * c->wsize;
}

template <typename T>
static int run_sweep_x(Context* c)
{
	SweepXArgs a {};
	a.field = c->field.ptr;
	a.coef = c->coef[0].ptr;
	a.coef_c = c->coef_c[0].ptr;
	a.coef_pitch = c->coef_pitch[0];
	a.n = c->n[0];
	a.pitch = c->pitch;
	a.rows = c->n[1] * c->n[2];
	a.rblocks = (a.rows + kSweepXRows - 1) / kSweepXRows;
	a.tiles = a.rblocks * c->S;
	a.smem_pitch = sweep_x_smem_pitch(c);
	a.err = static_cast<uint32_t*>(c->err.ptr);
	const uint64_t smem = sweep_x_smem_bytes(c);
	if (smem > kMaxSmemBytes)
		return fail(PCG_ERR_UNSUPPORTED, "x extent too long for the shared-memory x sweep");
	PCG_CUDA_TRY(cudaFuncSetAttribute(sweep_x_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	cudaEvent_t ev;
	launch_begin(c, K_SWEEP_X, 2.0 * (double)(c->V * c->S) * (double)sizeof(T), &ev);
	sweep_x_kernel<T><<<(unsigned)a.tiles, kSweepXRows, smem, c->stream>>>(a);
	launch_end(c, K_SWEEP_X, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

template <typename T>
static int run_sweep_yz(Context* c, int axis)
{
	SweepYZArgs a {};
	a.field = c->field.ptr;
	a.coef = c->coef[axis].ptr;
	a.coef_c = c->coef_c[axis].ptr;
	a.coef_pitch = c->coef_pitch[axis];
	a.n = c->n[axis];
	a.nx = c->n[0];
	a.plane = c->plane;
	if (axis == 1)
	{
		a.line_stride = c->pitch;
		a.outer_count = c->n[2];
		a.outer_stride = c->n[1] * c->pitch;
	}
	else
	{
		a.line_stride = c->n[1] * c->pitch;
		a.outer_count = c->n[1];
		a.outer_stride = c->pitch;
	}
	a.xblocks = (c->n[0] + kSweepLanes - 1) / kSweepLanes;
	a.tiles = a.xblocks * a.outer_count * c->S;
	a.err = static_cast<uint32_t*>(c->err.ptr);
	const uint64_t smem = sweep_yz_smem_bytes(c, axis);
	if (smem > kMaxSmemBytes)
		return fail(PCG_ERR_UNSUPPORTED, "line too long for the shared-memory y/z sweep");
	PCG_CUDA_TRY(cudaFuncSetAttribute(sweep_yz_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
	const int kid = axis == 1 ? K_SWEEP_Y : K_SWEEP_Z;
	cudaEvent_t ev;
	launch_begin(c, kid, 2.0 * (double)(c->V * c->S) * (double)sizeof(T), &ev);
	sweep_yz_kernel<T><<<(unsigned)a.tiles, kSweepLanes, smem, c->stream>>>(a);
	launch_end(c, kid, ev);
	PCG_CUDA_TRY(cudaGetLastError());
	return PCG_OK;
}

int launch_sweep_x(Context* c) { return c->wsize == 4 ? run_sweep_x<float>(c) : run_sweep_x<double>(c); }

int launch_sweep_yz(Context* c, int axis)
{
	return c->wsize == 4 ? run_sweep_yz<float>(c, axis) : run_sweep_yz<double>(c, axis);
}

} // namespace pcg
