// sweep_solvers.cuh -- per-line Thomas solvers shared by the single-domain and
// batched sweeps.  Arithmetic per line follows the reference
// (openmp_solver/src/diffusion_solver.cpp:116-202 and 390-794): forward
// d_i = d_i + e_{i-1} d_{i-1}, then d_i = (d_i + c d_{i+1}) b'_i downwards, both
// started from a zero carry (e_{-1} = 0; c*0 = 0 gives d_{n-1} b'_{n-1}).
#pragma once

#include "pcg_internal.cuh"

namespace pcg {
namespace solvers {

constexpr int kBlock = 8;      // recurrence steps per pipelined block (y/z, one point per step)
constexpr int kChunkBlock = 4; // 16-byte chunks per pipelined block (x, several points per chunk)

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

template <typename V, typename T>
__device__ __forceinline__ T vget(const V& v, int u)
{
	return reinterpret_cast<const T*>(&v)[u];
}
template <typename V, typename T>
__device__ __forceinline__ void vset(V& v, int u, T x)
{
	reinterpret_cast<T*>(&v)[u] = x;
}

template <typename V>
__device__ __forceinline__ V ldg_vec(const V* p)
{
	return __ldg(p);
}


// One line at col[j*kLanes], j < n, in shared memory; eE/eB are the line's
// substrate rows of a [s][j] coefficient table (16-byte aligned, padded to a
// multiple of kBlock).  Blocks of kBlock points are pipelined: the next block's
// points and coefficients are requested before the current block's chain.
template <typename T>
__device__ __forceinline__ void solve_column(T* __restrict__ col, uint32_t n, const T* __restrict__ eB,
											 const T* __restrict__ eE, T c)
{
	using V = typename Vec16<T>::type;
	constexpr int P = kBlock, VN = Vec16<T>::N, NV = P / VN;
	const uint32_t nb = n / P;
	T d = T(0);
	{
		T x[P], xn[P];
		V e[NV], en[NV];
		if (nb)
		{
#pragma unroll
			for (int q = 0; q < P; q++)
				x[q] = col[q * kLanes];
#pragma unroll
			for (int v = 0; v < NV; v++)
				e[v] = __ldg(reinterpret_cast<const V*>(eE) + v);
		}
		for (uint32_t b = 0; b < nb; b++)
		{
			T* blk = col + (uint64_t)b * P * kLanes;
			if (b + 1 < nb)
			{
#pragma unroll
				for (int q = 0; q < P; q++)
					xn[q] = blk[(P + q) * kLanes];
#pragma unroll
				for (int v = 0; v < NV; v++)
					en[v] = __ldg(reinterpret_cast<const V*>(eE + (b + 1) * P) + v);
			}
#pragma unroll
			for (int q = 0; q < P; q++)
			{
				d = dev::fmadd(vget<V, T>(e[q / VN], q % VN), d, x[q]);
				blk[q * kLanes] = d;
			}
#pragma unroll
			for (int q = 0; q < P; q++)
				x[q] = xn[q];
#pragma unroll
			for (int v = 0; v < NV; v++)
				e[v] = en[v];
		}
		for (uint32_t j = nb * P; j < n; j++)
		{
			d = dev::fmadd(__ldg(eE + j), d, col[(uint64_t)j * kLanes]);
			col[(uint64_t)j * kLanes] = d;
		}
	}
	d = T(0);
	for (int j = (int)n - 1; j >= (int)(nb * P); j--)
	{
		d = dev::fmadd(c, d, col[(uint64_t)j * kLanes]) * __ldg(eB + j);
		col[(uint64_t)j * kLanes] = d;
	}
	{
		T x[P], xn[P];
		V bb[NV], bn[NV];
		if (nb)
		{
			const T* blk = col + (uint64_t)(nb - 1) * P * kLanes;
#pragma unroll
			for (int q = 0; q < P; q++)
				x[q] = blk[q * kLanes];
#pragma unroll
			for (int v = 0; v < NV; v++)
				bb[v] = __ldg(reinterpret_cast<const V*>(eB + (nb - 1) * P) + v);
		}
		for (int b = (int)nb - 1; b >= 0; b--)
		{
			T* blk = col + (uint64_t)b * P * kLanes;
			if (b > 0)
			{
#pragma unroll
				for (int q = 0; q < P; q++)
					xn[q] = blk[(q - P) * kLanes];
#pragma unroll
				for (int v = 0; v < NV; v++)
					bn[v] = __ldg(reinterpret_cast<const V*>(eB + (b - 1) * P) + v);
			}
#pragma unroll
			for (int q = P - 1; q >= 0; q--)
			{
				d = dev::fmadd(c, d, x[q]) * vget<V, T>(bb[q / VN], q % VN);
				blk[q * kLanes] = d;
			}
#pragma unroll
			for (int q = 0; q < P; q++)
				x[q] = xn[q];
#pragma unroll
			for (int v = 0; v < NV; v++)
				bb[v] = bn[v];
		}
	}
}


// solve_column over a line whose points arrive in chunks of R points (R a
// multiple of kBlock): ready(ch) is called before chunk ch is first read, and
// done(ch) once back substitution has finished every point of chunk ch.  All
// lanes of the warp make the same calls, so the hooks may synchronise the warp.
template <typename T, typename Ready, typename Done>
__device__ __forceinline__ void solve_column_chunked(T* __restrict__ col, uint32_t n, uint32_t R,
													 const T* __restrict__ eB, const T* __restrict__ eE, T c,
													 Ready&& ready, Done&& done)
{
	using V = typename Vec16<T>::type;
	constexpr int P = kBlock, VN = Vec16<T>::N, NV = P / VN;
	const uint32_t nb = n / P, tail = n - nb * P;
	T d = T(0);
	ready(0u);
	{
		T x[P], xn[P];
		V e[NV], en[NV];
		if (nb)
		{
#pragma unroll
			for (int q = 0; q < P; q++)
				x[q] = col[q * kLanes];
#pragma unroll
			for (int v = 0; v < NV; v++)
				e[v] = __ldg(reinterpret_cast<const V*>(eE) + v);
		}
		for (uint32_t b = 0; b < nb; b++)
		{
			T* blk = col + (uint64_t)b * P * kLanes;
			if (b + 1 < nb)
			{
				if (((b + 1) * P) % R == 0)
					ready((b + 1) * P / R);
#pragma unroll
				for (int q = 0; q < P; q++)
					xn[q] = blk[(P + q) * kLanes];
#pragma unroll
				for (int v = 0; v < NV; v++)
					en[v] = __ldg(reinterpret_cast<const V*>(eE + (b + 1) * P) + v);
			}
#pragma unroll
			for (int q = 0; q < P; q++)
			{
				d = dev::fmadd(vget<V, T>(e[q / VN], q % VN), d, x[q]);
				blk[q * kLanes] = d;
			}
#pragma unroll
			for (int q = 0; q < P; q++)
				x[q] = xn[q];
#pragma unroll
			for (int v = 0; v < NV; v++)
				e[v] = en[v];
		}
		if (tail && nb && (nb * P) % R == 0)
			ready(nb * P / R);
		for (uint32_t j = nb * P; j < n; j++)
		{
			d = dev::fmadd(__ldg(eE + j), d, col[(uint64_t)j * kLanes]);
			col[(uint64_t)j * kLanes] = d;
		}
	}
	d = T(0);
	for (int j = (int)n - 1; j >= (int)(nb * P); j--)
	{
		d = dev::fmadd(c, d, col[(uint64_t)j * kLanes]) * __ldg(eB + j);
		col[(uint64_t)j * kLanes] = d;
	}
	if (tail && (nb * P) % R == 0)
		done(nb * P / R);
	{
		T x[P], xn[P];
		V bb[NV], bn[NV];
		if (nb)
		{
			const T* blk = col + (uint64_t)(nb - 1) * P * kLanes;
#pragma unroll
			for (int q = 0; q < P; q++)
				x[q] = blk[q * kLanes];
#pragma unroll
			for (int v = 0; v < NV; v++)
				bb[v] = __ldg(reinterpret_cast<const V*>(eB + (nb - 1) * P) + v);
		}
		for (int b = (int)nb - 1; b >= 0; b--)
		{
			T* blk = col + (uint64_t)b * P * kLanes;
			if (b > 0)
			{
#pragma unroll
				for (int q = 0; q < P; q++)
					xn[q] = blk[(q - P) * kLanes];
#pragma unroll
				for (int v = 0; v < NV; v++)
					bn[v] = __ldg(reinterpret_cast<const V*>(eB + (b - 1) * P) + v);
			}
#pragma unroll
			for (int q = P - 1; q >= 0; q--)
			{
				d = dev::fmadd(c, d, x[q]) * vget<V, T>(bb[q / VN], q % VN);
				blk[q * kLanes] = d;
			}
			if (((uint32_t)b * P) % R == 0)
				done((uint32_t)b * P / R);
#pragma unroll
			for (int q = 0; q < P; q++)
				x[q] = xn[q];
#pragma unroll
			for (int v = 0; v < NV; v++)
				bb[v] = bn[v];
		}
	}
}

// One substrate s of a row (stride S in shared memory): the substrate-per-thread
// mapping of the x sweep, with the same per-step arithmetic as the row solvers.
template <typename T>
__device__ __forceinline__ void solve_row_strided(T* row, const T* __restrict__ cB, const T* __restrict__ cE,
												  const T* __restrict__ cC, uint32_t n, uint32_t S, uint32_t s)
{
	constexpr int P = kBlock;
	T* __restrict__ r = row + s;
	const T* __restrict__ e = cE + s;
	const T* __restrict__ b = cB + s;
	const uint32_t nb = n / P;
	T d = T(0);
	for (uint32_t k = 0; k < nb; k++)
	{
		T x[P], ee[P];
#pragma unroll
		for (int q = 0; q < P; q++)
		{
			x[q] = r[(k * P + q) * S];
			ee[q] = __ldg(e + (k * P + q) * S);
		}
#pragma unroll
		for (int q = 0; q < P; q++)
		{
			d = dev::fmadd(ee[q], d, x[q]);
			r[(k * P + q) * S] = d;
		}
	}
	for (uint32_t i = nb * P; i < n; i++)
	{
		d = dev::fmadd(__ldg(e + i * S), d, r[i * S]);
		r[i * S] = d;
	}
	const T c = __ldg(cC + s);
	d = T(0);
	for (int i = (int)n - 1; i >= (int)(nb * P); i--)
	{
		d = dev::fmadd(c, d, r[i * S]) * __ldg(b + i * S);
		r[i * S] = d;
	}
	for (int k = (int)nb - 1; k >= 0; k--)
	{
		T x[P], bb[P];
#pragma unroll
		for (int q = 0; q < P; q++)
		{
			x[q] = r[(k * P + q) * S];
			bb[q] = __ldg(b + (k * P + q) * S);
		}
#pragma unroll
		for (int q = P - 1; q >= 0; q--)
		{
			d = dev::fmadd(c, d, x[q]) * bb[q];
			r[(k * P + q) * S] = d;
		}
	}
}

// S*sizeof(T) a multiple of 16 bytes: thread h of a row's TPR threads owns chunk
// slot h of every x position (VN substrates, VN independent recurrences).
template <typename T, int TPR>
__device__ __forceinline__ void solve_row_chunks(T* row, const T* __restrict__ cB, const T* __restrict__ cE,
												 const T* __restrict__ cC, uint32_t n, int h)
{
	using V = typename Vec16<T>::type;
	constexpr int VN = Vec16<T>::N, P = kChunkBlock;
	V* __restrict__ vrow = reinterpret_cast<V*>(row) + h;
	const V* vE = reinterpret_cast<const V*>(cE) + h;
	const V* vB = reinterpret_cast<const V*>(cB) + h;
	const uint32_t nb = n / P;
	T d[VN], c[VN];
#pragma unroll
	for (int u = 0; u < VN; u++)
	{
		d[u] = T(0);
		c[u] = __ldg(cC + h * VN + u);
	}
	auto step_fwd = [&](V& v, const V& e) {
#pragma unroll
		for (int u = 0; u < VN; u++)
		{
			d[u] = dev::fmadd(vget<V, T>(e, u), d[u], vget<V, T>(v, u));
			vset<V, T>(v, u, d[u]);
		}
	};
	auto step_bwd = [&](V& v, const V& b) {
#pragma unroll
		for (int u = 0; u < VN; u++)
		{
			d[u] = dev::fmadd(c[u], d[u], vget<V, T>(v, u)) * vget<V, T>(b, u);
			vset<V, T>(v, u, d[u]);
		}
	};
	{
		V x[P], xn[P], e[P], en[P];
		if (nb)
#pragma unroll
			for (int q = 0; q < P; q++)
			{
				x[q] = vrow[q * TPR];
				e[q] = ldg_vec(vE + q * TPR);
			}
		for (uint32_t b = 0; b < nb; b++)
		{
			const uint32_t i0 = b * P;
			if (b + 1 < nb)
#pragma unroll
				for (int q = 0; q < P; q++)
				{
					xn[q] = vrow[(i0 + P + q) * TPR];
					en[q] = ldg_vec(vE + (i0 + P + q) * TPR);
				}
#pragma unroll
			for (int q = 0; q < P; q++)
			{
				step_fwd(x[q], e[q]);
				vrow[(i0 + q) * TPR] = x[q];
			}
#pragma unroll
			for (int q = 0; q < P; q++)
			{
				x[q] = xn[q];
				e[q] = en[q];
			}
		}
		for (uint32_t i = nb * P; i < n; i++)
		{
			V v = vrow[i * TPR];
			step_fwd(v, ldg_vec(vE + i * TPR));
			vrow[i * TPR] = v;
		}
	}
#pragma unroll
	for (int u = 0; u < VN; u++)
		d[u] = T(0);
	for (int i = (int)n - 1; i >= (int)(nb * P); i--)
	{
		V v = vrow[i * TPR];
		step_bwd(v, ldg_vec(vB + i * TPR));
		vrow[i * TPR] = v;
	}
	{
		V x[P], xn[P], bb[P], bn[P];
		if (nb)
#pragma unroll
			for (int q = 0; q < P; q++)
			{
				x[q] = vrow[((nb - 1) * P + q) * TPR];
				bb[q] = ldg_vec(vB + ((nb - 1) * P + q) * TPR);
			}
		for (int b = (int)nb - 1; b >= 0; b--)
		{
			const uint32_t i0 = (uint32_t)b * P;
			if (b > 0)
#pragma unroll
				for (int q = 0; q < P; q++)
				{
					xn[q] = vrow[(i0 - P + q) * TPR];
					bn[q] = ldg_vec(vB + (i0 - P + q) * TPR);
				}
#pragma unroll
			for (int q = P - 1; q >= 0; q--)
			{
				step_bwd(x[q], bb[q]);
				vrow[(i0 + q) * TPR] = x[q];
			}
#pragma unroll
			for (int q = 0; q < P; q++)
			{
				x[q] = xn[q];
				bb[q] = bn[q];
			}
		}
	}
}

// ST substrates (1..8) not filling whole chunks: the row is a stream of chunks,
// element k of substrate k % ST.  Blocks of NB chunks hold whole groups of
// lcm(ST, VN) elements, so each element's substrate is a compile-time index.
template <typename T, int ST>
__device__ __forceinline__ void solve_row_vec(T* row, const T* __restrict__ cB, const T* __restrict__ cE,
											  const T* __restrict__ cC, uint32_t n)
{
	using V = typename Vec16<T>::type;
	constexpr int VN = Vec16<T>::N;
	constexpr int GE = group_elems(ST, VN);
	constexpr int U = GE / VN;
	constexpr int NB = U * ((kChunkBlock + U - 1) / U); // chunks per block
	const uint32_t total = n * ST;
	const uint32_t nchunks = (total + GE - 1) / GE * U; // whole groups (tail elements predicated)
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
	// In a block or group starting at chunk k0 (k0*VN a multiple of ST), element
	// k0*VN + q*VN + u has substrate (q*VN + u) % ST.
	auto fwd_chunk = [&](V& v, const V& e, int q, uint32_t k) {
#pragma unroll
		for (int u = 0; u < VN; u++)
		{
			const int s = (q * VN + u) % ST;
			if (k * VN + u < total)
			{
				d[s] = dev::fmadd(vget<V, T>(e, u), d[s], vget<V, T>(v, u));
				vset<V, T>(v, u, d[s]);
			}
		}
	};
	auto bwd_chunk = [&](V& v, const V& b, int q, uint32_t k) {
#pragma unroll
		for (int u = VN - 1; u >= 0; u--)
		{
			const int s = (q * VN + u) % ST;
			if (k * VN + u < total)
			{
				d[s] = dev::fmadd(c[s], d[s], vget<V, T>(v, u)) * vget<V, T>(b, u);
				vset<V, T>(v, u, d[s]);
			}
		}
	};
	const uint32_t nb = nchunks / NB;
	{
		V x[NB], xn[NB], e[NB], en[NB];
		if (nb)
#pragma unroll
			for (int q = 0; q < NB; q++)
			{
				x[q] = vrow[q];
				e[q] = ldg_vec(vE + q);
			}
		for (uint32_t b = 0; b < nb; b++)
		{
			const uint32_t k0 = b * NB;
			if (b + 1 < nb)
#pragma unroll
				for (int q = 0; q < NB; q++)
				{
					xn[q] = vrow[k0 + NB + q];
					en[q] = ldg_vec(vE + k0 + NB + q);
				}
#pragma unroll
			for (int q = 0; q < NB; q++)
			{
				fwd_chunk(x[q], e[q], q, k0 + q);
				vrow[k0 + q] = x[q];
			}
#pragma unroll
			for (int q = 0; q < NB; q++)
			{
				x[q] = xn[q];
				e[q] = en[q];
			}
		}
		// remaining whole groups (fewer than NB chunks)
		for (uint32_t k0 = nb * NB; k0 < nchunks; k0 += U)
		{
#pragma unroll
			for (int q = 0; q < U; q++)
			{
				V v = vrow[k0 + q];
				fwd_chunk(v, ldg_vec(vE + k0 + q), q, k0 + q);
				vrow[k0 + q] = v;
			}
		}
	}
#pragma unroll
	for (int s = 0; s < ST; s++)
		d[s] = T(0);
	for (int k0 = (int)nchunks - U; k0 >= (int)(nb * NB); k0 -= U)
	{
#pragma unroll
		for (int q = U - 1; q >= 0; q--)
		{
			V v = vrow[k0 + q];
			bwd_chunk(v, ldg_vec(vB + k0 + q), q, (uint32_t)(k0 + q));
			vrow[k0 + q] = v;
		}
	}
	{
		V x[NB], xn[NB], bb[NB], bn[NB];
		if (nb)
#pragma unroll
			for (int q = 0; q < NB; q++)
			{
				x[q] = vrow[(nb - 1) * NB + q];
				bb[q] = ldg_vec(vB + (nb - 1) * NB + q);
			}
		for (int b = (int)nb - 1; b >= 0; b--)
		{
			const uint32_t k0 = (uint32_t)b * NB;
			if (b > 0)
#pragma unroll
				for (int q = 0; q < NB; q++)
				{
					xn[q] = vrow[k0 - NB + q];
					bn[q] = ldg_vec(vB + k0 - NB + q);
				}
#pragma unroll
			for (int q = NB - 1; q >= 0; q--)
			{
				bwd_chunk(x[q], bb[q], q, k0 + q);
				vrow[k0 + q] = x[q];
			}
#pragma unroll
			for (int q = 0; q < NB; q++)
			{
				x[q] = xn[q];
				bb[q] = bn[q];
			}
		}
	}
}

// Any S: one recurrence at a time, scalar shared-memory accesses.
template <typename T>
__device__ __forceinline__ void solve_row_generic(T* row, const T* cB, const T* cE, const T* cC, uint32_t n,
												  uint32_t S)
{
	for (uint32_t s = 0; s < S; s++)
	{
		T d = T(0);
		for (uint32_t i = 0; i < n; i++)
		{
			d = dev::fmadd(__ldg(cE + i * S + s), d, row[i * S + s]);
			row[i * S + s] = d;
		}
		const T c = __ldg(cC + s);
		d = T(0);
		for (int i = (int)n - 1; i >= 0; i--)
		{
			d = dev::fmadd(c, d, row[i * S + s]) * __ldg(cB + i * S + s);
			row[i * S + s] = d;
		}
	}
}

template <typename T, int ST>
constexpr int x_tpr()
{
	return (ST > 0 && ST <= 8 && (ST * (int)sizeof(T)) % 16 == 0) ? ST * (int)sizeof(T) / 16 : 1;
}


// Solves one x row of substrate count S at compile time when S <= 8.
template <typename T, int ST>
__device__ __forceinline__ void solve_row(T* row, const T* cB, const T* cE, const T* cC, uint32_t n, uint32_t S, int h)
{
	if constexpr (ST == 0)
		solve_row_generic<T>(row, cB, cE, cC, n, S);
	else if constexpr ((ST * (int)sizeof(T)) % 16 == 0)
		solve_row_chunks<T, x_tpr<T, ST>()>(row, cB, cE, cC, n, h);
	else
		solve_row_vec<T, ST>(row, cB, cE, cC, n);
}

} // namespace solvers
} // namespace pcg
