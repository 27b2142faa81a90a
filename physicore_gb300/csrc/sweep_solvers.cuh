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

// Mass-check accumulators: a lane's running total of the values a sweep reads
// (before the step's first sweep) or writes (after its last sweep), fused into
// the solvers so the check needs no pass of its own.  FP32: a float pair
// hi + lo accumulated with Knuth's TwoSum (error-free), fed with FP32 sums of
// blocks of points, so about one extra instruction per point; FP64: a double.
template <typename T>
struct MassAcc;

template <>
struct MassAcc<float>
{
	float hi, lo;
	__device__ __forceinline__ void zero() { hi = lo = 0.f; }
	__device__ __forceinline__ void add(float x)
	{
		const float s = __fadd_rn(hi, x);
		const float bb = __fsub_rn(s, hi);
		lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(x, bb)));
		hi = s;
	}
	template <int P>
	__device__ __forceinline__ void add_block(const float (&x)[P])
	{
		static_assert(P == 8, "blocks of 8 points");
		add(__fadd_rn(__fadd_rn(__fadd_rn(x[0], x[1]), __fadd_rn(x[2], x[3])),
					  __fadd_rn(__fadd_rn(x[4], x[5]), __fadd_rn(x[6], x[7]))));
	}
	__device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

template <>
struct MassAcc<double>
{
	double v;
	__device__ __forceinline__ void zero() { v = 0.0; }
	__device__ __forceinline__ void add(double x) { v += x; }
	template <int P>
	__device__ __forceinline__ void add_block(const double (&x)[P])
	{
		static_assert(P == 8, "blocks of 8 points");
		v += ((x[0] + x[1]) + (x[2] + x[3])) + ((x[4] + x[5]) + (x[6] + x[7]));
	}
	__device__ __forceinline__ double value() const { return v; }
};

// Mass-check modes of a solver call (bits): sum the inputs, sum the outputs.
enum : int
{
	kMcIn = 1,
	kMcOut = 2,
};

// Adds the totals v of the first `width` lanes of the warp to FP64 totals with
// atomics, where lanes l and l + stride (stride <= 32) add to the same total: the
// classes are summed by a tree over strides stride, 2*stride, ..., then lane
// l < stride adds its class's sum to *dst (its own target).  All `width` lanes
// of the warp call it.
__device__ __forceinline__ void flush_classes(double v, uint32_t stride, uint32_t width, double* dst)
{
	const uint32_t lane = threadIdx.x & 31;
	const uint32_t mask = width >= 32 ? 0xffffffffu : ((1u << width) - 1u);
	for (uint32_t k = stride; k < 32; k <<= 1)
	{
		const double t = __shfl_down_sync(mask, v, k);
		if (lane + k < width)
			v += t;
	}
	if (lane < stride && lane < width && v != 0.0)
		atomicAdd(dst, v);
}

// One lane's coefficients along a line, from the compressed tables of an axis:
// points j < H read the substrate's head rows, points H <= j < n-1 share the middle
// constants, and point n-1 has its own (when H >= n the head holds the whole line).
// H is a multiple of kBlock, so a block of points is either all head or all
// middle/last.  The stored values are the full table's (the host picks H so that
// every point from H to n-2 holds exactly the middle value).
template <typename T>
struct LineCoef
{
	const T* hB;
	const T* hE;
	const T* hBl; // FP32: lo parts of the multipliers (head rows), null for FP64
	uint32_t H, n;
	T mB, mE, lB, lE, c;
	T mBl, lBl; // FP32: lo parts of the middle and last multipliers
};

// One backward step d = (x + c d) b'.  FP32: evaluated as d = (b' c) d + b' x, with
// the FP32 coupling b' c = RN(bh * c) and the product b' x taken with the
// multiplier's pair bh + lo (the host's column-sum-exact multipliers account for
// the coupling's rounding), so the chain from one point to the next is a single
// fma (b' x does not depend on the chain).  FP64 tables hold b' itself (lo
// unused) and keep the reference's form.
__device__ __forceinline__ float bwd_step(float c, float d, float x, float bh, float bl)
{
	const float bc = bh * c;
	const float xb = dev::fmadd(x, bh, x * bl);
	return dev::fmadd(bc, d, xb);
}
__device__ __forceinline__ double bwd_step(double c, double d, double x, double bh, double)
{
	return dev::fmadd(c, d, x) * bh;
}

// Compressed table of an axis: [head b' (S x H) | head e (S x H) | mid b' | mid e |
// last b' | last e | c], the five constant arrays kS = S rounded up to 16 bytes long;
// FP32 tables continue with [head b' lo (S x H) | mid b' lo | last b' lo].
template <typename T>
__device__ __forceinline__ LineCoef<T> line_coef(const T* comp, uint32_t S, uint32_t H, uint32_t n, uint32_t s)
{
	constexpr uint32_t VN = 16 / sizeof(T);
	const uint32_t kS = (S + VN - 1) / VN * VN;
	const T* k = comp + 2ull * S * H;
	LineCoef<T> L;
	L.hB = comp + (uint64_t)s * H;
	L.hE = comp + (uint64_t)S * H + (uint64_t)s * H;
	L.H = H;
	L.n = n;
	L.mB = __ldg(k + s);
	L.mE = __ldg(k + kS + s);
	L.lB = __ldg(k + 2 * kS + s);
	L.lE = __ldg(k + 3 * kS + s);
	L.c = __ldg(k + 4 * kS + s);
	if constexpr (sizeof(T) == 4)
	{
		const T* lo = k + 5 * kS;
		L.hBl = lo + (uint64_t)s * H;
		L.mBl = __ldg(lo + (uint64_t)S * H + s);
		L.lBl = __ldg(lo + (uint64_t)S * H + kS + s);
	}
	else
	{
		L.hBl = nullptr;
		L.mBl = L.lBl = T(0);
	}
	return L;
}

template <typename T>
__device__ __forceinline__ T coef_at(const T* head, uint32_t H, T mid, T last, uint32_t n, uint32_t j)
{
	return j < H ? __ldg(head + j) : (j == n - 1 ? last : mid);
}

// One line of n points at col[j * stride] in shared memory (stride = STRIDE, or the
// run-time value when STRIDE is 0) with the lane's coefficients L.  The line is
// three runs: head blocks of kBlock points [0, hb) (coefficients from the head
// rows), middle blocks [hb, q) (the middle constants, held in registers) and the
// points from q * kBlock on, which hold point n-1 (coefficients chosen per point;
// at most 2 kBlock - 1 of them).  Within a run the next block's points (and head
// coefficients) are requested before the current block's dependent chain, so
// their latency overlaps it; the middle run, nearly the whole line, alternates two
// register sets, so that its blocks carry no copies or tests.  Which run a block
// is in is the same for every lane of a warp (one n and H per launch).
//
// MC (kMcIn / kMcOut bits) adds the line's input values to *acc_in and its
// solved values to *acc_out.
template <typename T, int STRIDE, int MC = 0>
__device__ __forceinline__ void solve_line(T* __restrict__ col, uint32_t n, uint32_t rt_stride, const LineCoef<T>& L,
										   MassAcc<T>* acc_in = nullptr, MassAcc<T>* acc_out = nullptr)
{
	using V = typename Vec16<T>::type;
	constexpr int P = kBlock, VN = Vec16<T>::N, NV = P / VN;
	constexpr bool kLo = sizeof(T) == 4;
	const uint32_t st = STRIDE ? (uint32_t)STRIDE : rt_stride;
	const uint32_t nb = n / P;
	const uint32_t hb = min(L.H / P, nb);
	const uint32_t q = max((n - 1) / P, hb); // blocks [hb, q) have j0 >= H and j0 + P <= n - 1
	const T c = L.c;
	// the middle coupling of the backward step, as bwd_step forms it per point
	const T mbc = kLo ? L.mB * c : T(0);
	// offsets within the tile stay far below 2^32
	auto load = [&](uint32_t b, T(&x)[P]) {
		const T* blk = col + b * (uint32_t)P * st;
#pragma unroll
		for (int k = 0; k < P; k++)
			x[k] = blk[k * st];
	};
	auto fetch_head = [&](const T* head, uint32_t b, V(&out)[NV]) {
#pragma unroll
		for (int v = 0; v < NV; v++)
			out[v] = __ldg(reinterpret_cast<const V*>(head + b * P) + v);
	};
	T d = T(0);

	// ---- forward elimination
	auto fwd_mid = [&](uint32_t b, const T(&x)[P]) {
		T* blk = col + b * (uint32_t)P * st;
		if constexpr ((MC & kMcIn) != 0)
			acc_in->add_block(x);
#pragma unroll
		for (int k = 0; k < P; k++)
		{
			d = dev::fmadd(L.mE, d, x[k]);
			blk[k * st] = d;
		}
	};
	if (hb)
	{
		T x[P], xn[P];
		V e[NV], en[NV];
		load(0, x);
		fetch_head(L.hE, 0, e);
		for (uint32_t b = 0; b < hb; b++)
		{
			if (b + 1 < hb)
			{
				load(b + 1, xn);
				fetch_head(L.hE, b + 1, en);
			}
			if constexpr ((MC & kMcIn) != 0)
				acc_in->add_block(x);
			T* blk = col + b * (uint32_t)P * st;
#pragma unroll
			for (int k = 0; k < P; k++)
			{
				d = dev::fmadd(vget<V, T>(e[k / VN], k % VN), d, x[k]);
				blk[k * st] = d;
			}
#pragma unroll
			for (int k = 0; k < P; k++)
				x[k] = xn[k];
#pragma unroll
			for (int v = 0; v < NV; v++)
				e[v] = en[v];
		}
	}
	if (hb < q)
	{
		T xa[P], xb[P];
		uint32_t b = hb;
		load(b, xa);
		for (; b + 2 < q; b += 2)
		{
			load(b + 1, xb);
			fwd_mid(b, xa);
			load(b + 2, xa);
			fwd_mid(b + 1, xb);
		}
		if (b + 1 < q)
		{
			load(b + 1, xb);
			fwd_mid(b, xa);
			fwd_mid(b + 1, xb);
		}
		else
			fwd_mid(b, xa);
	}
	for (uint32_t j = q * P; j < n; j++)
	{
		const T xj = col[j * st];
		if constexpr ((MC & kMcIn) != 0)
			acc_in->add(xj);
		d = dev::fmadd(coef_at(L.hE, L.H, L.mE, L.lE, n, j), d, xj);
		col[j * st] = d;
	}

	// ---- back substitution
	d = T(0);
	for (int j = (int)n - 1; j >= (int)(q * P); j--)
	{
		const T bl = kLo ? coef_at(L.hBl, L.H, L.mBl, L.lBl, n, (uint32_t)j) : T(0);
		d = bwd_step(c, d, col[(uint32_t)j * st], coef_at(L.hB, L.H, L.mB, L.lB, n, (uint32_t)j), bl);
		col[(uint32_t)j * st] = d;
		if constexpr ((MC & kMcOut) != 0)
			acc_out->add(d);
	}
	auto bwd_mid = [&](uint32_t b, const T(&x)[P]) {
		T* blk = col + b * (uint32_t)P * st;
		T y[P];
#pragma unroll
		for (int k = P - 1; k >= 0; k--)
		{
			if constexpr (kLo)
				d = dev::fmadd(mbc, d, dev::fmadd(x[k], L.mB, x[k] * L.mBl));
			else
				d = dev::fmadd(c, d, x[k]) * L.mB;
			blk[k * st] = d;
			y[k] = d;
		}
		if constexpr ((MC & kMcOut) != 0)
			acc_out->add_block(y);
	};
	if (hb < q)
	{
		T xa[P], xb[P];
		uint32_t b = q - 1;
		load(b, xa);
		for (; b >= hb + 2; b -= 2)
		{
			load(b - 1, xb);
			bwd_mid(b, xa);
			load(b - 2, xa);
			bwd_mid(b - 1, xb);
		}
		if (b >= hb + 1)
		{
			load(b - 1, xb);
			bwd_mid(b, xa);
			bwd_mid(b - 1, xb);
		}
		else
			bwd_mid(b, xa);
	}
	if (hb)
	{
		T x[P], xn[P];
		V bb[NV], bn[NV], bl[NV], bln[NV];
		load(hb - 1, x);
		fetch_head(L.hB, hb - 1, bb);
		if constexpr (kLo)
			fetch_head(L.hBl, hb - 1, bl);
		for (int b = (int)hb - 1; b >= 0; b--)
		{
			if (b > 0)
			{
				load((uint32_t)b - 1, xn);
				fetch_head(L.hB, (uint32_t)b - 1, bn);
				if constexpr (kLo)
					fetch_head(L.hBl, (uint32_t)b - 1, bln);
			}
			T* blk = col + (uint32_t)b * (uint32_t)P * st;
			T y[P];
#pragma unroll
			for (int k = P - 1; k >= 0; k--)
			{
				d = bwd_step(c, d, x[k], vget<V, T>(bb[k / VN], k % VN), kLo ? vget<V, T>(bl[k / VN], k % VN) : T(0));
				blk[k * st] = d;
				y[k] = d;
			}
			if constexpr ((MC & kMcOut) != 0)
				acc_out->add_block(y);
#pragma unroll
			for (int k = 0; k < P; k++)
				x[k] = xn[k];
#pragma unroll
			for (int v = 0; v < NV; v++)
			{
				bb[v] = bn[v];
				if constexpr (kLo)
					bl[v] = bln[v];
			}
		}
	}
}

// S*sizeof(T) a multiple of 16 bytes: thread h of a row's TPR threads owns chunk
// slot h of every x position (VN substrates, VN independent recurrences).
// MC adds element u's inputs / outputs to acc_in[u] / acc_out[u] (substrate h*VN + u).
// cBl: the FP32 multipliers' lo parts (same layout as cB), null for FP64.
template <typename T, int TPR, int MC = 0>
__device__ __forceinline__ void solve_row_chunks(T* row, const T* __restrict__ cB, const T* __restrict__ cE,
												 const T* __restrict__ cC, const T* __restrict__ cBl, uint32_t n, int h,
												 MassAcc<T>* acc_in = nullptr, MassAcc<T>* acc_out = nullptr)
{
	using V = typename Vec16<T>::type;
	constexpr int VN = Vec16<T>::N, P = kChunkBlock;
	constexpr bool kLo = sizeof(T) == 4;
	V* __restrict__ vrow = reinterpret_cast<V*>(row) + h;
	const V* vE = reinterpret_cast<const V*>(cE) + h;
	const V* vB = reinterpret_cast<const V*>(cB) + h;
	const V* vBl = kLo ? reinterpret_cast<const V*>(cBl) + h : nullptr;
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
			if constexpr ((MC & kMcIn) != 0)
				acc_in[u].add(vget<V, T>(v, u));
			d[u] = dev::fmadd(vget<V, T>(e, u), d[u], vget<V, T>(v, u));
			vset<V, T>(v, u, d[u]);
		}
	};
	auto step_bwd = [&](V& v, const V& b, const V& bl) {
#pragma unroll
		for (int u = 0; u < VN; u++)
		{
			d[u] = bwd_step(c[u], d[u], vget<V, T>(v, u), vget<V, T>(b, u), kLo ? vget<V, T>(bl, u) : T(0));
			vset<V, T>(v, u, d[u]);
			if constexpr ((MC & kMcOut) != 0)
				acc_out[u].add(d[u]);
		}
	};
	auto ldg_lo = [&](uint32_t k) {
		V z {};
		if constexpr (kLo)
			z = ldg_vec(vBl + k);
		return z;
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
		step_bwd(v, ldg_vec(vB + i * TPR), ldg_lo(i * TPR));
		vrow[i * TPR] = v;
	}
	{
		V x[P], xn[P], bb[P], bn[P], bl[P], bln[P];
		if (nb)
#pragma unroll
			for (int q = 0; q < P; q++)
			{
				x[q] = vrow[((nb - 1) * P + q) * TPR];
				bb[q] = ldg_vec(vB + ((nb - 1) * P + q) * TPR);
				bl[q] = ldg_lo(((nb - 1) * P + q) * TPR);
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
					bln[q] = ldg_lo((i0 - P + q) * TPR);
				}
#pragma unroll
			for (int q = P - 1; q >= 0; q--)
			{
				step_bwd(x[q], bb[q], bl[q]);
				vrow[(i0 + q) * TPR] = x[q];
			}
#pragma unroll
			for (int q = 0; q < P; q++)
			{
				x[q] = xn[q];
				bb[q] = bn[q];
				bl[q] = bln[q];
			}
		}
	}
}

// ST substrates (1..8) not filling whole chunks: the row is a stream of chunks,
// element k of substrate k % ST.  Blocks of NB chunks hold whole groups of
// lcm(ST, VN) elements, so each element's substrate is a compile-time index.  The
// blocks that lie wholly inside the row run without per-element tests, two
// register sets in turn (the next block's chunks and coefficients load while the
// current block's chain runs, and no block is copied from one set to the other);
// the chunks after them, at most NB + U - 1, test each element against the row's
// end.  MC adds substrate s's inputs / outputs to acc_in[s] / acc_out[s].
template <typename T, int ST, int MC = 0>
__device__ __forceinline__ void solve_row_vec(T* row, const T* __restrict__ cB, const T* __restrict__ cE,
											  const T* __restrict__ cC, const T* __restrict__ cBl, uint32_t n,
											  MassAcc<T>* acc_in = nullptr, MassAcc<T>* acc_out = nullptr)
{
	using V = typename Vec16<T>::type;
	constexpr int VN = Vec16<T>::N;
	constexpr int GE = group_elems(ST, VN);
	constexpr int U = GE / VN;
	constexpr int NB = U * ((kChunkBlock + U - 1) / U); // chunks per block
	const uint32_t total = n * ST;
	const uint32_t nchunks = (total + GE - 1) / GE * U; // whole groups (tail elements tested)
	const uint32_t nfull = total / (NB * VN);           // blocks wholly inside the row
	constexpr bool kLo = sizeof(T) == 4;
	V* __restrict__ vrow = reinterpret_cast<V*>(row);
	const V* vE = reinterpret_cast<const V*>(cE);
	const V* vB = reinterpret_cast<const V*>(cB);
	const V* vBl = reinterpret_cast<const V*>(cBl);
	auto ldg_lo = [&](uint32_t k) {
		V z {};
		if constexpr (kLo)
			z = ldg_vec(vBl + k);
		return z;
	};
	T d[ST], c[ST];
#pragma unroll
	for (int s = 0; s < ST; s++)
	{
		d[s] = T(0);
		c[s] = __ldg(cC + s);
	}
	// In a block or group starting at chunk k0 (k0*VN a multiple of ST), element
	// k0*VN + q*VN + u has substrate (q*VN + u) % ST.  TEST: check the element
	// against the row's end.
	auto fwd_chunk = [&](V& v, const V& e, int q, uint32_t k, bool test) {
#pragma unroll
		for (int u = 0; u < VN; u++)
		{
			const int s = (q * VN + u) % ST;
			if (!test || k * VN + u < total)
			{
				if constexpr ((MC & kMcIn) != 0)
					acc_in[s].add(vget<V, T>(v, u));
				d[s] = dev::fmadd(vget<V, T>(e, u), d[s], vget<V, T>(v, u));
				vset<V, T>(v, u, d[s]);
			}
		}
	};
	auto bwd_chunk = [&](V& v, const V& b, const V& bl, int q, uint32_t k, bool test) {
#pragma unroll
		for (int u = VN - 1; u >= 0; u--)
		{
			const int s = (q * VN + u) % ST;
			if (!test || k * VN + u < total)
			{
				d[s] = bwd_step(c[s], d[s], vget<V, T>(v, u), vget<V, T>(b, u), kLo ? vget<V, T>(bl, u) : T(0));
				vset<V, T>(v, u, d[s]);
				if constexpr ((MC & kMcOut) != 0)
					acc_out[s].add(d[s]);
			}
		}
	};

	// ---- forward elimination
	auto fwd_load = [&](uint32_t b, V(&x)[NB], V(&e)[NB]) {
#pragma unroll
		for (int q = 0; q < NB; q++)
		{
			x[q] = vrow[b * NB + q];
			e[q] = ldg_vec(vE + b * NB + q);
		}
	};
	auto fwd_block = [&](uint32_t b, V(&x)[NB], const V(&e)[NB]) {
#pragma unroll
		for (int q = 0; q < NB; q++)
		{
			fwd_chunk(x[q], e[q], q, b * NB + q, false);
			vrow[b * NB + q] = x[q];
		}
	};
	if (nfull)
	{
		V xa[NB], ea[NB], xb[NB], eb[NB];
		uint32_t b = 0;
		fwd_load(0, xa, ea);
		for (; b + 2 < nfull; b += 2)
		{
			fwd_load(b + 1, xb, eb);
			fwd_block(b, xa, ea);
			fwd_load(b + 2, xa, ea);
			fwd_block(b + 1, xb, eb);
		}
		if (b + 1 < nfull)
		{
			fwd_load(b + 1, xb, eb);
			fwd_block(b, xa, ea);
			fwd_block(b + 1, xb, eb);
		}
		else
			fwd_block(b, xa, ea);
	}
	for (uint32_t k0 = nfull * NB; k0 < nchunks; k0 += U)
	{
#pragma unroll
		for (int q = 0; q < U; q++)
		{
			V v = vrow[k0 + q];
			fwd_chunk(v, ldg_vec(vE + k0 + q), q, k0 + q, true);
			vrow[k0 + q] = v;
		}
	}

	// ---- back substitution
#pragma unroll
	for (int s = 0; s < ST; s++)
		d[s] = T(0);
	for (int k0 = (int)nchunks - U; k0 >= (int)(nfull * NB); k0 -= U)
	{
#pragma unroll
		for (int q = U - 1; q >= 0; q--)
		{
			V v = vrow[k0 + q];
			bwd_chunk(v, ldg_vec(vB + k0 + q), ldg_lo(k0 + q), q, (uint32_t)(k0 + q), true);
			vrow[k0 + q] = v;
		}
	}
	auto bwd_load = [&](uint32_t b, V(&x)[NB], V(&bb)[NB], V(&bl)[NB]) {
#pragma unroll
		for (int q = 0; q < NB; q++)
		{
			x[q] = vrow[b * NB + q];
			bb[q] = ldg_vec(vB + b * NB + q);
			bl[q] = ldg_lo(b * NB + q);
		}
	};
	auto bwd_block = [&](uint32_t b, V(&x)[NB], const V(&bb)[NB], const V(&bl)[NB]) {
#pragma unroll
		for (int q = NB - 1; q >= 0; q--)
		{
			bwd_chunk(x[q], bb[q], bl[q], q, b * NB + q, false);
			vrow[b * NB + q] = x[q];
		}
	};
	if (nfull)
	{
		V xa[NB], ba[NB], la[NB], xb[NB], bbb[NB], lb[NB];
		uint32_t b = nfull - 1;
		bwd_load(b, xa, ba, la);
		for (; b >= 2; b -= 2)
		{
			bwd_load(b - 1, xb, bbb, lb);
			bwd_block(b, xa, ba, la);
			bwd_load(b - 2, xa, ba, la);
			bwd_block(b - 1, xb, bbb, lb);
		}
		if (b >= 1)
		{
			bwd_load(b - 1, xb, bbb, lb);
			bwd_block(b, xa, ba, la);
			bwd_block(b - 1, xb, bbb, lb);
		}
		else
			bwd_block(b, xa, ba, la);
	}
}

// Any S: one recurrence at a time, scalar shared-memory accesses.  MC adds
// substrate s's input / output total of the row to mc_in[s] / mc_out[s] (FP64
// atomics per row; a path for rare substrate counts).
template <typename T, int MC = 0>
__device__ __forceinline__ void solve_row_generic(T* row, const T* cB, const T* cE, const T* cC, const T* cBl,
												  uint32_t n, uint32_t S, double* mc_in = nullptr,
												  double* mc_out = nullptr)
{
	for (uint32_t s = 0; s < S; s++)
	{
		MassAcc<T> ai, ao;
		ai.zero();
		ao.zero();
		T d = T(0);
		for (uint32_t i = 0; i < n; i++)
		{
			if constexpr ((MC & kMcIn) != 0)
				ai.add(row[i * S + s]);
			d = dev::fmadd(__ldg(cE + i * S + s), d, row[i * S + s]);
			row[i * S + s] = d;
		}
		const T c = __ldg(cC + s);
		d = T(0);
		for (int i = (int)n - 1; i >= 0; i--)
		{
			d = bwd_step(c, d, row[i * S + s], __ldg(cB + i * S + s), sizeof(T) == 4 ? __ldg(cBl + i * S + s) : T(0));
			row[i * S + s] = d;
			if constexpr ((MC & kMcOut) != 0)
				ao.add(d);
		}
		if constexpr ((MC & kMcIn) != 0)
			if (mc_in)
				atomicAdd(mc_in + s, ai.value());
		if constexpr ((MC & kMcOut) != 0)
			if (mc_out)
				atomicAdd(mc_out + s, ao.value());
	}
}

template <typename T, int ST>
constexpr int x_tpr()
{
	return (ST > 0 && ST <= 8 && (ST * (int)sizeof(T)) % 16 == 0) ? ST * (int)sizeof(T) / 16 : 1;
}


// Solves one x row of substrate count S at compile time when S <= 8.
template <typename T, int ST>
__device__ __forceinline__ void solve_row(T* row, const T* cB, const T* cE, const T* cC, const T* cBl, uint32_t n,
										  uint32_t S, int h)
{
	if constexpr (ST == 0)
		solve_row_generic<T>(row, cB, cE, cC, cBl, n, S);
	else if constexpr ((ST * (int)sizeof(T)) % 16 == 0)
		solve_row_chunks<T, x_tpr<T, ST>()>(row, cB, cE, cC, cBl, n, h);
	else
		solve_row_vec<T, ST>(row, cB, cE, cC, cBl, n);
}

} // namespace solvers
} // namespace pcg
