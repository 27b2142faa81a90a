// capi.cu -- the extern "C" surface of include/physicore_gb300.h.
//
// The context owns every device buffer of one BioFVM problem and queues all work
// on one CUDA stream.  Step orchestration follows openmp_solver::solve
// (openmp_solver.cpp:23-40): diffusion (x, then y and z when the mesh has them,
// diffusion_solver.cpp:797-843), Dirichlet, bulk, cells; the ballot is rebuilt on
// every iteration of a solve call that follows initialize or
// recompute_positional_data, and the flag is cleared when the call returns.
#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>

#include "pcg_internal.cuh"

namespace pcg {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg)
{
	set_error(msg);
	return code;
}

const char* kernel_name(int id)
{
	static const char* names[K_COUNT] = { "sweep_x",	  "sweep_y",		"sweep_z",	   "dirichlet_faces",
										  "dirichlet_interior", "bulk", "cells_locate", "cells_ballot",
										  "cells_reduce", "cells_apply", "cells_internalize", "cells_release",
										  "mass",		  "layout", "cells_clear", "mass_check", "cells_group",
										  "sweep_xy" };
	return (id >= 0 && id < K_COUNT) ? names[id] : "?";
}

// The library's stream-ordered memory pool on a device.  A block freed on one
// stream is handed to an allocation on another only once that free has completed
// on the device (no cross-stream dependency is inserted), so an allocation never
// waits for other contexts' queued work; a server admitting requests while its
// batched steps run is not held up by them.  Up to kPoolKeepBytes of freed blocks
// stay in the pool for reuse (beyond that they go back to the device at the next
// synchronisation); the pool's idle bytes count as free to a server's admission.
constexpr uint64_t kPoolKeepBytes = 4ull << 30;
static std::mutex g_pool_mu;
static std::map<int, cudaMemPool_t> g_pools;

static cudaMemPool_t library_pool(int device)
{
	std::lock_guard<std::mutex> lk(g_pool_mu);
	auto it = g_pools.find(device);
	if (it != g_pools.end())
		return it->second;
	cudaMemPoolProps props {};
	props.allocType = cudaMemAllocationTypePinned;
	props.handleTypes = cudaMemHandleTypeNone;
	props.location.type = cudaMemLocationTypeDevice;
	props.location.id = device;
	cudaMemPool_t pool = nullptr;
	if (cudaMemPoolCreate(&pool, &props) != cudaSuccess)
	{
		cudaGetLastError();
		return nullptr;
	}
	int off = 0, on = 1;
	uint64_t keep = kPoolKeepBytes;
	cudaMemPoolSetAttribute(pool, cudaMemPoolReuseFollowEventDependencies, &off);
	cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &off);
	cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowOpportunistic, &on);
	cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
	cudaGetLastError();
	g_pools[device] = pool;
	return pool;
}

cudaError_t pool_alloc(void** ptr, size_t bytes, cudaStream_t stream, int device)
{
	cudaMemPool_t pool = library_pool(device);
	return pool ? cudaMallocFromPoolAsync(ptr, bytes, pool, stream) : cudaMallocAsync(ptr, bytes, stream);
}

uint64_t pool_idle_bytes(int device)
{
	cudaMemPool_t pool;
	{
		std::lock_guard<std::mutex> lk(g_pool_mu);
		auto it = g_pools.find(device);
		if (it == g_pools.end())
			return 0;
		pool = it->second;
	}
	uint64_t reserved = 0, used = 0;
	if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) != cudaSuccess ||
		cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) != cudaSuccess)
	{
		cudaGetLastError();
		return 0;
	}
	return reserved > used ? reserved - used : 0;
}

static std::mutex g_words_mu;
static std::vector<uint32_t*> g_free_words;

uint32_t* pinned_words_get()
{
	std::lock_guard<std::mutex> lk(g_words_mu);
	if (g_free_words.empty())
	{
		constexpr size_t kUnits = 1024; // 16 KB of pinned memory, four words a unit, never freed
		uint32_t* blk = nullptr;
		if (cudaHostAlloc(reinterpret_cast<void**>(&blk), kUnits * 4 * sizeof(uint32_t), cudaHostAllocDefault) !=
			cudaSuccess)
		{
			cudaGetLastError();
			return nullptr;
		}
		for (size_t u = 0; u < kUnits; u++)
			g_free_words.push_back(blk + 4 * u);
	}
	uint32_t* w = g_free_words.back();
	g_free_words.pop_back();
	return w;
}

void pinned_words_put(uint32_t* w)
{
	if (!w)
		return;
	std::lock_guard<std::mutex> lk(g_words_mu);
	g_free_words.push_back(w);
}

// Waits for the context's stream with the calling thread asleep (a blocking-sync
// event) rather than spinning: a thread spinning in a stream synchronisation slows
// the CUDA calls of other threads in the process -- a server's admissions and
// steps -- while it waits, which can be milliseconds when the stream's kernels
// queue behind other work on the SMs.
cudaError_t stream_wait(Context* c)
{
	if (!c->ev_block)
	{
		cudaError_t e = cudaEventCreateWithFlags(&c->ev_block, cudaEventBlockingSync | cudaEventDisableTiming);
		if (e != cudaSuccess)
		{
			c->ev_block = nullptr;
			return e;
		}
	}
	cudaError_t e = cudaEventRecord(c->ev_block, c->stream);
	return e != cudaSuccess ? e : cudaEventSynchronize(c->ev_block);
}

// Context buffers come from the library's pool on the context's own stream, which
// lives as long as the context; freeing them (a replaced buffer, or pcg_destroy)
// then never synchronises the device, so a process that creates and destroys many
// contexts while others run (a server) does not stall them.
int dalloc(Context* c, DeviceBuffer& b, size_t bytes)
{
	if (b.ptr && b.bytes >= bytes)
		return PCG_OK;
	if (b.ptr)
	{
		stream_wait(c); // earlier work may still read the old buffer
		dfree(b);
	}
	if (bytes == 0)
		return PCG_OK;
	cudaStream_t s = c->own_stream;
	const size_t span = round_up(bytes, 256);
	if (c->slab.ptr && span <= c->slab.bytes - c->slab_used)
	{
		b.ptr = static_cast<char*>(c->slab.ptr) + c->slab_used;
		b.bytes = bytes;
		b.stream = c->slab.stream;
		b.carved = true;
		c->slab_used += span;
		return PCG_OK; // ordered like the slab's own allocation
	}
	cudaError_t e = s ? pool_alloc(&b.ptr, bytes, s, c->device) : cudaMalloc(&b.ptr, bytes);
	if (e != cudaSuccess)
	{
		b.ptr = nullptr;
		cudaGetLastError();
		return fail(PCG_ERR_NOMEM, "device allocation of " + std::to_string(bytes) + " bytes failed: " +
									   cudaGetErrorString(e));
	}
	b.bytes = bytes;
	b.stream = s;
	// Work on the context's stream is ordered after the allocation when that stream
	// is the own stream (the usual case, and always under a server; batches wait for
	// it through events).  A caller-set stream is not: wait for the allocation.
	if (s && s != c->stream)
		cudaStreamSynchronize(s);
	return PCG_OK;
}

void dfree(DeviceBuffer& b)
{
	if (b.ptr && !b.carved)
	{
		if (b.stream)
			cudaFreeAsync(b.ptr, b.stream);
		else
			cudaFree(b.ptr);
	}
	b.ptr = nullptr;
	b.bytes = 0;
	b.stream = nullptr;
	b.carved = false;
}

static cudaEvent_t get_event(Context* c)
{
	if (!c->event_pool.empty())
	{
		cudaEvent_t e = c->event_pool.back();
		c->event_pool.pop_back();
		return e;
	}
	cudaEvent_t e = nullptr;
	cudaEventCreate(&e);
	return e;
}

void launch_begin(Context* c, int kid, double bytes, cudaEvent_t* ev)
{
	c->launches++;
	c->stats[kid].launches++;
	c->stats[kid].bytes += bytes;
	*ev = nullptr;
	if (c->timing)
	{
		*ev = get_event(c);
		cudaEventRecord(*ev, c->stream);
	}
}

void launch_end(Context* c, int kid, cudaEvent_t ev, double per_shared, double per_writer)
{
	if (!c->timing || !ev)
		return;
	cudaEvent_t stop = get_event(c);
	cudaEventRecord(stop, c->stream);
	c->pending.push_back({ kid, ev, stop, per_shared, per_writer });
}

// In timing mode the cell step copies the number of agents in shared voxels and
// of agents that write a voxel to pinned words after every ballot; launches whose
// work is those agents add their bytes per agent times those numbers once their
// events have completed.
void collect_timings(Context* c)
{
	if (!c->pending.empty() && c->h_words)
	{
		cudaEventSynchronize(c->pending.back().b);
		c->shared_agents = c->h_words[2];
		c->writer_agents = c->h_words[3];
	}
	for (auto& p : c->pending)
	{
		cudaEventSynchronize(p.b);
		float ms = 0;
		cudaEventElapsedTime(&ms, p.a, p.b);
		c->stats[p.kid].total_ms += ms;
		c->stats[p.kid].bytes += p.per_shared * c->shared_agents + p.per_writer * c->writer_agents;
		c->event_pool.push_back(p.a);
		c->event_pool.push_back(p.b);
	}
	c->pending.clear();
}

// ------------------------------------------------------------------ helpers

// Reads and clears the device error word after synchronising the stream.
std::string device_error_text(uint32_t word)
{
	std::string msg = "device fault:";
	if (word & DEV_ERR_AGENT_OUTSIDE)
		msg += " an active agent lies outside the mesh;";
	if (word & DEV_ERR_WAIT_TIMEOUT)
		msg += " a bounded shared-memory wait timed out;";
	if (word & DEV_ERR_DIRICHLET_INDEX)
		msg += " a Dirichlet voxel lies outside the mesh;";
	if (word & DEV_ERR_BAD_TILE)
		msg += " a batched tile descriptor was invalid;";
	return msg;
}

static int check_device(Context* c)
{
	if (!c->err.ptr)
		return PCG_OK; // nothing has run on the device yet
	if (!c->h_words && !(c->h_words = pinned_words_get()))
		return fail(PCG_ERR_NOMEM, "pinned host memory for the device error word");
	// The copy is queued only once the stream is idle: a copy waiting in a copy
	// engine's queue for kernels (which may wait for other work to leave the SMs)
	// holds up the copies other threads queue behind it.
	cudaError_t e = stream_wait(c);
	if (e != cudaSuccess)
		return fail(PCG_ERR_CUDA, std::string("stream synchronise: ") + cudaGetErrorString(e));
	PCG_CUDA_TRY(cudaMemcpyAsync(c->h_words, c->err.ptr, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
	PCG_CUDA_TRY(stream_wait(c));
	collect_timings(c);
	const uint32_t word = c->h_words[0];
	if (word)
	{
		PCG_CUDA_TRY(cudaMemsetAsync(c->err.ptr, 0, sizeof(uint32_t), c->stream));
		return fail(PCG_ERR_DEVICE, device_error_text(word));
	}
	return PCG_OK;
}

// diffusion_solver::precompute_values (openmp_solver/src/diffusion_solver.cpp:29-86),
// evaluated in FP64 for one axis.  Outputs b'[i*S+s], e[(i-1)*S+s], c[s].
static void precompute_axis(uint64_t n, uint64_t S, uint64_t shape, uint64_t dims, double dt, const double* D,
							const double* decay, std::vector<double>& b, std::vector<double>& e,
							std::vector<double>& cc)
{
	const double h2 = (double)(shape * shape);
	b.assign(n * S, 0.0);
	e.assign((n > 0 ? n - 1 : 0) * S, 0.0);
	cc.assign(S, 0.0);
	for (uint64_t s = 0; s < S; s++)
		cc[s] = -1 * -dt * D[s] / h2; // c = dt*D/h^2 (the reference stores -a_i)
	for (uint64_t i = 0; i < n; i++)
		for (uint64_t s = 0; s < S; s++)
		{
			double v = 1 + decay[s] * dt / (double)dims + 2 * dt * D[s] / h2;
			if (i == 0 || i == n - 1) // Neumann rows; a single subtraction when n == 1
				v -= dt * D[s] / h2;
			b[i * S + s] = v;
		}
	for (uint64_t s = 0; s < S; s++)
		b[s] = 1 / b[s];
	for (uint64_t i = 1; i < n; i++)
		for (uint64_t s = 0; s < S; s++)
		{
			b[i * S + s] = 1 / (b[i * S + s] - cc[s] * cc[s] * b[(i - 1) * S + s]);
			e[(i - 1) * S + s] = cc[s] * b[(i - 1) * S + s];
		}
}

// FP32 backward multipliers that keep the sweep's mass exact.  The FP32 solve uses
// E = e and c rounded to FP32 and evaluates each backward step as
// d_i = B_i x_i + K_i d_{i+1}, with the coupling K_i = RN32(RN32(B_i) c) and B_i
// applied as a pair hi + lo (sweep_solvers.cuh, bwd_step).  The tridiagonal matrix
// this factorisation inverts is M' = L'U', L'[i][i-1] = -E[i-1], U'[i][i] = 1/B_i,
// U'[i][i+1] = -K_i/B_i =: -C'_i, whose column j sums to
// (1 - E[j]) / B[j] - (1 - E[j-1]) C'[j-1] (E[-1] = C'[-1] = 0, E[n-1] = 0).
// Choosing B[j] in FP64, in order, so that every column sums exactly to the
// reference matrix's column sum (diffusion_solver.cpp:29-86: the diagonal minus r
// for each neighbour) makes M' conserve mass exactly as the reference does; with
// the exact e and c it gives b'[j] itself.  Plain FP32 rounding of b', e and c
// otherwise biases every step the same way, and over hundreds of steps that drift
// dominates the FP32 error.
static void colsum_multipliers(uint64_t n, uint64_t S, uint64_t shape, uint64_t dims, double dt, const double* D,
							   const double* decay, const std::vector<double>& e, const std::vector<double>& cc,
							   std::vector<double>& B, std::vector<float>& Bhi)
{
	const double h2 = (double)(shape * shape);
	B.assign(n * S, 0.0);
	Bhi.assign(n * S, 0.0f);
	for (uint64_t s = 0; s < S; s++)
	{
		const double r = dt * D[s] / h2;
		const float C32 = (float)cc[s];
		auto kappa = [&](uint64_t j) {
			double diag = 1 + decay[s] * dt / (double)dims + 2 * dt * D[s] / h2;
			if (j == 0 || j == n - 1)
				diag -= dt * D[s] / h2;
			return diag - (j > 0 ? r : 0.0) - (j + 1 < n ? r : 0.0);
		};
		auto E = [&](int64_t j) { return j >= 0 && (uint64_t)j + 1 < n ? (double)(float)e[j * S + s] : 0.0; };
		auto K = [&](float hi) {
			const volatile float k = hi * C32; // the device's FP32 product
			return (double)k;
		};
		double Cp = 0.0; // C'[j-1]
		for (uint64_t j = 0; j < n; j++)
		{
			const double b = (1.0 - E(j)) / (kappa(j) + (1.0 - E((int64_t)j - 1)) * Cp);
			B[j * S + s] = b;
			Bhi[j * S + s] = (float)b;
			Cp = K((float)b) / b;
		}
		if (n < 3)
			continue;
		// The middle: FP32 rounding of B feeds back through the coupling, so the
		// sequence can settle into a two-value cycle instead of a constant.  The
		// middle instead takes the hi part Bh of the last middle value, the coupling
		// K = RN32(Bh c) and the exact fixed point (1 - E)(1 - K) / kappa of the
		// column-sum condition, stored as Bh + lo (lo may span a few ulps of Bh);
		// the sequence hands over to it at the first point whose predecessor has
		// the same hi part and lies within 1e-7 of it (that one column's sum is then
		// off by at most about 1e-7; every other column is exact).
		const double Em = E((int64_t)n - 3);
		const float Bh = (float)B[(n - 2) * S + s];
		const double Km = K(Bh);
		const double Bmid = (1.0 - Em) * (1.0 - Km) / kappa(n - 2);
		for (uint64_t j = 1; j + 1 < n; j++)
		{
			if (E(j) != Em || E((int64_t)j - 1) != Em || Bhi[(j - 1) * S + s] != Bh ||
				!(std::fabs(B[(j - 1) * S + s] / Bmid - 1.0) < 1e-7))
				continue;
			for (uint64_t k = j; k + 1 < n; k++)
			{
				B[k * S + s] = Bmid;
				Bhi[k * S + s] = Bh;
			}
			const double bl = 1.0 / (kappa(n - 1) + (1.0 - E((int64_t)n - 2)) * Km / Bmid);
			B[(n - 1) * S + s] = bl;
			Bhi[(n - 1) * S + s] = (float)bl;
			break;
		}
	}
}

// Device coefficient table of one axis: [B | E | C], C[s] = c.  For x, B and E are
// flat in the field's (i, s) order, B[i*S+s] = b'_i, E[i*S+s] = e_{i-1} (0 at i = 0),
// so a 16-byte chunk of coefficients matches a chunk of a row.  For y and z they are
// per-substrate rows, B[s*cp + i], padded to cp = a multiple of the solver block.
// FP32 tables hold the column-sum-exact multipliers as hi + lo (colsum_multipliers):
// B is the hi part and a B_lo table of the same layout follows C.
template <typename T>
static int upload_coefficients(Context* c)
{
	const uint64_t S = c->S;
	constexpr bool kLo = sizeof(T) == 4;
	for (int axis = 0; axis < c->dims; axis++)
	{
		const uint64_t n = c->n[axis];
		std::vector<double> b, e, cc, B;
		std::vector<float> Bhi;
		precompute_axis(n, S, c->voxel[axis], (uint64_t)c->dims, c->dt, c->D.data(), c->decay.data(), b, e, cc);
		if (kLo)
		{
			colsum_multipliers(n, S, c->voxel[axis], (uint64_t)c->dims, c->dt, c->D.data(), c->decay.data(), e, cc,
							   B, Bhi);
			b = B;
		}
		// FP32: the multiplier's hi part (chosen by colsum_multipliers) and lo = B - hi
		auto hi = [&](uint64_t k) { return kLo ? (T)Bhi[k] : (T)b[k]; };
		auto lo = [&](uint64_t k) { return kLo ? (T)(b[k] - (double)Bhi[k]) : T(0); };
		const uint64_t cp = coef_row_pitch(n);
		const uint64_t len = axis == 0 ? coef_table_len(n, S, sizeof(T)) : S * cp;
		const uint64_t blo_off = 2 * len + round_up(S, 16 / sizeof(T));
		const uint64_t total = blo_off + (kLo ? len : 0);
		// Compressed tables.  b'_i and e_i converge to a constant within a few
		// points, so a line needs only a head of H points (the first index from which
		// every stored value up to n-2 equals the value at n-2, rounded up to the solver
		// block and taken over all substrates), that middle constant and the values of
		// the last point.  Stored values are the same rounded numbers as the full table.
		const uint64_t vn = 16 / sizeof(T);
		uint64_t H = 0;
		{
			for (uint64_t sub = 0; sub < S; sub++)
			{
				uint64_t h = n;
				if (n >= 2)
				{
					const T bm = hi((n - 2) * S + sub);
					const T em = n >= 3 ? (T)e[(n - 3) * S + sub] : T(0);
					h = n - 2;
					const T blm = lo((n - 2) * S + sub);
					while (h > 0)
					{
						const uint64_t i = h - 1;
						const T bi = hi(i * S + sub);
						const T ei = i == 0 ? T(0) : (T)e[(i - 1) * S + sub];
						if (bi != bm || ei != em || lo(i * S + sub) != blm)
							break;
						h = i;
					}
				}
				H = std::max(H, h);
			}
			H = round_up(std::max<uint64_t>(H, 1), kBlockPoints);
			if (H >= n)
				H = round_up(n, kBlockPoints); // the whole line lives in the head
		}
		const uint64_t kS = round_up(S, vn);
		const uint64_t comp_total = 2 * S * H + 5 * kS + (kLo ? S * H + 2 * kS : 0);
		c->coef_len[axis] = len;
		c->coef_elems[axis] = total;
		c->coef_comp_off[axis] = total;
		c->coef_blo_off[axis] = kLo ? blo_off : 0;
		c->coef_head[axis] = (uint32_t)H;
		std::vector<T> tab(total + comp_total, T(0));
		for (uint64_t i = 0; i < n; i++)
			for (uint64_t s = 0; s < S; s++)
			{
				const uint64_t at = axis == 0 ? i * S + s : s * cp + i;
				tab[at] = hi(i * S + s);
				tab[len + at] = i == 0 ? T(0) : (T)e[(i - 1) * S + s];
				if (kLo)
					tab[blo_off + at] = lo(i * S + s);
			}
		for (uint64_t s = 0; s < S; s++)
			tab[2 * len + s] = (T)cc[s];
		{
			T* hB = tab.data() + total;
			T* hE = hB + S * H;
			T* k = hE + S * H; // [mid b' | mid e | last b' | last e | c], each kS long
			T* hBl = k + 5 * kS; // FP32: [head b' lo | mid b' lo | last b' lo]
			T* kl = hBl + S * H;
			for (uint64_t sub = 0; sub < S; sub++)
			{
				for (uint64_t i = 0; i < std::min(H, n); i++)
				{
					hB[sub * H + i] = hi(i * S + sub);
					hE[sub * H + i] = i == 0 ? T(0) : (T)e[(i - 1) * S + sub];
					if (kLo)
						hBl[sub * H + i] = lo(i * S + sub);
				}
				const uint64_t m = n >= 2 ? n - 2 : 0;
				k[sub] = hi(m * S + sub);
				k[kS + sub] = m == 0 ? T(0) : (T)e[(m - 1) * S + sub];
				k[2 * kS + sub] = hi((n - 1) * S + sub);
				k[3 * kS + sub] = n == 1 ? T(0) : (T)e[(n - 2) * S + sub];
				k[4 * kS + sub] = (T)cc[sub];
				if (kLo)
				{
					kl[sub] = lo(m * S + sub);
					kl[kS + sub] = lo((n - 1) * S + sub);
				}
			}
		}
		int rc = dalloc(c, c->coef[axis], tab.size() * sizeof(T));
		if (rc)
			return rc;
		PCG_CUDA_TRY(cudaMemcpyAsync(c->coef[axis].ptr, tab.data(), tab.size() * sizeof(T), cudaMemcpyHostToDevice,
									 c->stream));
		PCG_CUDA_TRY(stream_wait(c)); // the host table dies at scope exit
	}
	return PCG_OK;
}

template <typename T>
static int upload_dirichlet(Context* c)
{
	const uint64_t S = c->S;
	int rc;
	// faces
	std::vector<T> fv(6 * S, T(0));
	std::vector<uint8_t> fc(6 * S, 0);
	for (int axis = 0; axis < 3; axis++)
		for (int side = 0; side < 2; side++)
			if (c->face_on[axis][side])
				for (uint64_t s = 0; s < S; s++)
				{
					fv[(axis * 2 + side) * S + s] = (T)c->h_face_values[axis][side][s];
					fc[(axis * 2 + side) * S + s] = c->h_face_conds[axis][side][s] ? 1 : 0;
				}
	if ((rc = dalloc(c, c->face_values, fv.size() * sizeof(T))))
		return rc;
	if ((rc = dalloc(c, c->face_conds, fc.size())))
		return rc;
	PCG_CUDA_TRY(cudaMemcpyAsync(c->face_values.ptr, fv.data(), fv.size() * sizeof(T), cudaMemcpyHostToDevice,
								 c->stream));
	PCG_CUDA_TRY(cudaMemcpyAsync(c->face_conds.ptr, fc.data(), fc.size(), cudaMemcpyHostToDevice, c->stream));
	// interior
	std::vector<uint64_t> off(c->K);
	std::vector<T> iv(c->K * S);
	std::vector<uint8_t> ic(c->K * S);
	for (uint64_t k = 0; k < c->K; k++)
	{
		uint64_t idx[3] = { 0, 0, 0 };
		for (int d = 0; d < c->dims; d++)
			idx[d] = c->h_dir_voxels[k * c->dims + d];
		off[k] = (idx[2] * c->n[1] + idx[1]) * c->pitch + idx[0] * S;
		for (uint64_t s = 0; s < S; s++)
		{
			iv[k * S + s] = (T)c->h_dir_values[k * S + s];
			ic[k * S + s] = c->h_dir_conds[k * S + s] ? 1 : 0;
		}
	}
	if (c->K)
	{
		if ((rc = dalloc(c, c->dir_offsets, off.size() * sizeof(uint64_t))))
			return rc;
		if ((rc = dalloc(c, c->dir_values, iv.size() * sizeof(T))))
			return rc;
		if ((rc = dalloc(c, c->dir_conds, ic.size())))
			return rc;
		PCG_CUDA_TRY(cudaMemcpyAsync(c->dir_offsets.ptr, off.data(), off.size() * sizeof(uint64_t),
									 cudaMemcpyHostToDevice, c->stream));
		PCG_CUDA_TRY(cudaMemcpyAsync(c->dir_values.ptr, iv.data(), iv.size() * sizeof(T), cudaMemcpyHostToDevice,
									 c->stream));
		PCG_CUDA_TRY(cudaMemcpyAsync(c->dir_conds.ptr, ic.data(), ic.size(), cudaMemcpyHostToDevice, c->stream));
	}
	PCG_CUDA_TRY(stream_wait(c));
	return PCG_OK;
}

// Bulk tables: [S] (uniform) or shaped like the field (per voxel, interleaved rows)
// from the host's planar [s][z][y][x] arrays.
template <typename T>
static int upload_bulk(Context* c)
{
	if (c->bulk_mode == PCG_BULK_NONE)
		return PCG_OK;
	const bool pv = c->bulk_mode == PCG_BULK_PER_VOXEL;
	const uint64_t cnt = pv ? c->rows * c->pitch : c->S;
	std::vector<T> tab(cnt, T(0));
	for (int k = 0; k < 3; k++)
	{
		if (pv)
		{
			const uint64_t nx = c->n[0], rows = c->rows, S = c->S;
			for (uint64_t s = 0; s < S; s++)
				for (uint64_t r = 0; r < rows; r++)
					for (uint64_t x = 0; x < nx; x++)
						tab[r * c->pitch + x * S + s] = (T)c->h_bulk[k][(s * rows + r) * nx + x];
		}
		else
			for (uint64_t s = 0; s < c->S; s++)
				tab[s] = (T)c->h_bulk[k][s];
		int rc = dalloc(c, c->bulk[k], cnt * sizeof(T));
		if (rc)
			return rc;
		PCG_CUDA_TRY(cudaMemcpyAsync(c->bulk[k].ptr, tab.data(), cnt * sizeof(T), cudaMemcpyHostToDevice, c->stream));
		PCG_CUDA_TRY(stream_wait(c)); // the host table dies at scope exit
	}
	return PCG_OK;
}

static int run_phases(Context* c, uint32_t phases, bool recompute)
{
	int rc;
	// with both phases in this call, the last sweep writes the boundary faces into
	// its tiles before storing them (the reference's next step, dirichlet_solver.cpp:
	// 59-83), which saves a pass of scattered writes
	// With the mass check on, the x sweep adds up its inputs and the last sweep its
	// outputs (before writing any face), so the check reads no extra field pass.
	const bool check = c->mass_check && (phases & PCG_PHASE_DIFFUSION);
	const bool fuse = (phases & PCG_PHASE_DIFFUSION) && (phases & PCG_PHASE_DIRICHLET) && faces_fusable(c);
	if (phases & PCG_PHASE_DIFFUSION)
	{
		if (xy_fusable(c))
		{
			if ((rc = launch_sweep_xy(c, check)))
				return rc;
		}
		else
		{
			if ((rc = launch_sweep_x(c, check)))
				return rc;
			if (c->dims >= 2 && (rc = launch_sweep_yz(c, 1, fuse && c->dims == 2, check && c->dims == 2)))
				return rc;
		}
		if (c->dims >= 3 && (rc = launch_sweep_yz(c, 2, fuse, check)))
			return rc;
		if (check && (rc = launch_mass_check_finish(c)))
			return rc;
		c->mass_checked_steps += check;
	}
	if ((phases & PCG_PHASE_DIRICHLET) && (rc = launch_dirichlet(c, fuse)))
		return rc;
	if ((phases & PCG_PHASE_BULK) && (rc = launch_bulk(c)))
		return rc;
	if ((phases & PCG_PHASE_CELLS) && (rc = launch_cells(c, recompute)))
		return rc;
	return PCG_OK;
}

// Row geometry of the interleaved field: a row holds nx*S elements and is padded
// to a multiple of 32 bytes.
static int derive_layout(Context* c)
{
	c->row_len = c->n[0] * c->S;
	c->pitch = round_up(c->row_len, 32 / c->wsize);
	c->rows = c->n[1] * c->n[2];
	if (c->rows * c->pitch >= 0xffffffffull)
		return fail(PCG_ERR_UNSUPPORTED, "fields beyond 2^32 elements are not supported");
	return PCG_OK;
}

int upload_agents(Context* c, uint64_t A, const double* positions, const double* secretion, const double* saturation,
				  const double* uptake, const double* net_export, const double* volumes, const uint8_t* is_active,
				  const double* internalized, const double* fraction_released, bool compute_internalized);

// The context's own stream and device words, created on first use.  With
// defer_clear the words are allocated but not yet cleared (no device work is
// queued): initialisation clears them after its host-blocking uploads.
int ensure_device_state(Context* c, bool defer_clear = false)
{
	if (!c->own_stream)
	{
		if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess)
		{
			c->own_stream = nullptr;
			cudaGetLastError();
			return fail(PCG_ERR_CUDA, "cudaStreamCreate failed");
		}
		if (!c->stream)
			c->stream = c->own_stream;
	}
	if (!c->err.ptr)
	{
		int rc = dalloc(c, c->err, sizeof(uint32_t) * 4);
		if (!rc)
			rc = dalloc(c, c->flags, sizeof(uint32_t) * 8);
		if (!rc)
			rc = dalloc(c, c->tickets, sizeof(uint32_t) * 4);
		if (rc)
			return rc;
		c->words_cleared = false;
	}
	if (!c->words_cleared && !defer_clear)
	{
		PCG_CUDA_TRY(cudaMemsetAsync(c->err.ptr, 0, sizeof(uint32_t) * 4, c->stream));
		PCG_CUDA_TRY(cudaMemsetAsync(c->flags.ptr, 0, sizeof(uint32_t) * 8, c->stream));
		c->words_cleared = true;
	}
	return PCG_OK;
}

// The initial values as T in the mass buffer (S doubles hold S T's), for the fill.
template <typename T>
static int upload_initial_values(Context* c)
{
	std::vector<T> h(c->S);
	for (uint64_t s = 0; s < c->S; s++)
		h[s] = (T)c->init[s];
	PCG_CUDA_TRY(cudaMemcpyAsync(c->mass.ptr, h.data(), c->S * sizeof(T), cudaMemcpyHostToDevice, c->stream));
	PCG_CUDA_TRY(stream_wait(c)); // the host vector dies at scope exit
	return PCG_OK;
}

// Allocations and uploads first: the host waits for each upload while the
// context's stream holds nothing else, so no wait depends on other work on the
// device.  The kernels (word clearing, field fill, ballot counts) come last.  With
// wait = false the call returns without waiting for them (a server admitting a
// request while its batched steps occupy the device); the next batch step orders
// them first, and a device error surfaces there.
static int do_initialize(Context* c, bool wait = true)
{
	if (c->initialized)
		return PCG_OK;
	{
		DeviceGuard g(c->device);
		const int rc0 = ensure_device_state(c, true);
		if (rc0)
			return rc0;
	}
	if (!c->mesh_set || c->S == 0)
		return fail(PCG_ERR_INVALID, "mesh and substrates must be set before initialize");
	int rc;
	if ((rc = derive_layout(c)))
		return rc;
	if (!c->slab.ptr)
	{
		const size_t bytes = estimate_device_bytes(c) + (64 << 10); // + alignment of the pieces
		if ((rc = dalloc(c, c->slab, bytes)))
			return rc;
		c->slab_used = 0;
	}
	if ((rc = dalloc(c, c->field, c->rows * c->pitch * c->wsize)))
		return rc;
	if ((rc = prepare_sweep_maps(c)))
		return rc;
	if ((rc = dalloc(c, c->mass, std::max<uint64_t>(c->S, 2) * sizeof(double))))
		return rc;
	rc = c->wsize == 4 ? upload_initial_values<float>(c) : upload_initial_values<double>(c);
	if (rc)
		return rc;
	rc = c->wsize == 4 ? upload_coefficients<float>(c) : upload_coefficients<double>(c);
	if (rc)
		return rc;
	rc = c->wsize == 4 ? upload_dirichlet<float>(c) : upload_dirichlet<double>(c);
	if (rc)
		return rc;
	rc = c->wsize == 4 ? upload_bulk<float>(c) : upload_bulk<double>(c);
	if (rc)
		return rc;
	// shared-memory feasibility of the sweeps, checked once here
	for (int axis = 0; axis < c->dims; axis++)
		if (sweep_smem_bytes(c, axis) > kMaxSmemBytes)
			return fail(PCG_ERR_UNSUPPORTED, "a line of axis " + std::to_string(axis) +
												 " exceeds the shared-memory sweep limit");
	if (c->staged_agents)
	{
		const Context::HostAgents& h = *c->staged_agents;
		rc = upload_agents(c, c->A, h.pos.data(), h.sec.data(), h.sat.data(), h.upt.data(), h.net.data(),
						   h.vol.data(), h.active.data(), h.internal.empty() ? nullptr : h.internal.data(),
						   h.frac.empty() ? nullptr : h.frac.data(), c->compute_internalized);
		if (rc)
			return rc;
		c->staged_agents.reset();
	}
	if ((rc = ensure_device_state(c)) || (rc = launch_fill_initial(c)))
		return rc;
	c->initialized = true;
	c->generation++;
	return wait ? check_device(c) : PCG_OK;
}

int initialize_context(Context* c, bool wait) { return do_initialize(c, wait); }
int check_context(Context* c) { return check_device(c); }

static int alloc_agents(Context* c, uint64_t A)
{
	const uint64_t S = c->S;
	int rc;
	const size_t w = c->wsize;
	DeviceBuffer* f64[] = { &c->a_sec, &c->a_sat, &c->a_upt, &c->a_net, &c->a_internal, &c->a_frac };
	for (DeviceBuffer* b : f64)
		if ((rc = dalloc(c, *b, std::max<uint64_t>(A * S, 1) * sizeof(double))))
			return rc;
	if ((rc = dalloc(c, c->a_pos, std::max<uint64_t>(A * c->dims, 1) * sizeof(double))))
		return rc;
	if ((rc = dalloc(c, c->a_vol, std::max<uint64_t>(A, 1) * sizeof(double))))
		return rc;
	if ((rc = dalloc(c, c->a_active, std::max<uint64_t>(A, 1))))
		return rc;
	if ((rc = dalloc(c, c->a_foff, std::max<uint64_t>(A, 1) * sizeof(uint32_t))))
		return rc;
	if ((rc = dalloc(c, c->a_vox, std::max<uint64_t>(A, 1) * sizeof(uint32_t))))
		return rc;
	if ((rc = dalloc(c, c->a_role, std::max<uint64_t>(A, 1))))
		return rc;
	if ((rc = dalloc(c, c->a_shared, std::max<uint64_t>(A, 1) * sizeof(uint32_t))))
		return rc;
	if ((rc = dalloc(c, c->a_rank, std::max<uint64_t>(A, 1) * sizeof(uint32_t))))
		return rc;
	if ((rc = dalloc(c, c->a_writers, std::max<uint64_t>(A, 1) * sizeof(uint32_t))))
		return rc;
	if ((rc = dalloc(c, c->a_sorted, std::max<uint64_t>(A, 1) * 2 * sizeof(uint32_t))))
		return rc;
	c->term_stride = term_stride(S, w);
	for (DeviceBuffer* b : { &c->a_terms, &c->a_reduced })
		if ((rc = dalloc(c, *b, std::max<uint64_t>(A * c->term_stride, 1) * w)))
			return rc;
	if ((rc = dalloc(c, c->owner, c->V * sizeof(uint32_t))))
		return rc;
	if ((rc = dalloc(c, c->counts, c->V * sizeof(uint32_t))))
		return rc;
	return PCG_OK;
}

// FP32 contexts hold internalized amounts as pairs of floats hi + lo in the 8 bytes
// of each double (hi first; cells_device.cuh, pair_add); conversions at the API.
static void to_pairs(const double* in, std::vector<double>& out, size_t n)
{
	out.resize(n);
	for (size_t k = 0; k < n; k++)
	{
		const float hi = (float)in[k];
		const float lo = (float)(in[k] - (double)hi);
		std::memcpy(reinterpret_cast<char*>(&out[k]), &hi, sizeof(float));
		std::memcpy(reinterpret_cast<char*>(&out[k]) + sizeof(float), &lo, sizeof(float));
	}
}

static void from_pairs(double* buf, size_t n)
{
	for (size_t k = 0; k < n; k++)
	{
		float hi, lo;
		std::memcpy(&hi, reinterpret_cast<const char*>(&buf[k]), sizeof(float));
		std::memcpy(&lo, reinterpret_cast<const char*>(&buf[k]) + sizeof(float), sizeof(float));
		buf[k] = (double)hi + (double)lo;
	}
}

int upload_agents(Context* c, uint64_t A, const double* positions, const double* secretion, const double* saturation,
				  const double* uptake, const double* net_export, const double* volumes, const uint8_t* is_active,
				  const double* internalized, const double* fraction_released, bool compute_internalized)
{
	int rc = alloc_agents(c, A);
	if (rc)
		return rc;
	c->A = A;
	c->compute_internalized = compute_internalized;
	const uint64_t S = c->S;
	if (A)
	{
		PCG_CUDA_TRY(cudaMemcpyAsync(c->a_pos.ptr, positions, A * c->dims * sizeof(double), cudaMemcpyHostToDevice,
									 c->stream));
		const double* rates[4] = { secretion, saturation, uptake, net_export };
		DeviceBuffer* dst[4] = { &c->a_sec, &c->a_sat, &c->a_upt, &c->a_net };
		for (int k = 0; k < 4; k++)
			PCG_CUDA_TRY(cudaMemcpyAsync(dst[k]->ptr, rates[k], A * S * sizeof(double), cudaMemcpyHostToDevice,
										 c->stream));
		PCG_CUDA_TRY(cudaMemcpyAsync(c->a_vol.ptr, volumes, A * sizeof(double), cudaMemcpyHostToDevice, c->stream));
		PCG_CUDA_TRY(cudaMemcpyAsync(c->a_active.ptr, is_active, A, cudaMemcpyHostToDevice, c->stream));
		std::vector<double> pairs;
		if (internalized && c->wsize == 4)
		{
			to_pairs(internalized, pairs, A * S);
			internalized = pairs.data(); // lives until the wait below
		}
		if (internalized)
			PCG_CUDA_TRY(cudaMemcpyAsync(c->a_internal.ptr, internalized, A * S * sizeof(double),
										 cudaMemcpyHostToDevice, c->stream));
		if (fraction_released)
			PCG_CUDA_TRY(cudaMemcpyAsync(c->a_frac.ptr, fraction_released, A * S * sizeof(double),
										 cudaMemcpyHostToDevice, c->stream));
		PCG_CUDA_TRY(stream_wait(c)); // the caller may free its arrays on return
		// device-side clears after the host wait, which then waits for copies only
		if (!internalized)
			PCG_CUDA_TRY(cudaMemsetAsync(c->a_internal.ptr, 0, A * S * sizeof(double), c->stream));
		if (!fraction_released)
			PCG_CUDA_TRY(cudaMemsetAsync(c->a_frac.ptr, 0, A * S * sizeof(double), c->stream));
		PCG_CUDA_TRY(cudaMemsetAsync(c->counts.ptr, 0, c->V * sizeof(uint32_t), c->stream));
	}
	c->recompute_cells = true;
	c->terms_dirty = true;
	return PCG_OK;
}

// Field, coefficient tables, error/flag/ticket words, Dirichlet and bulk tables,
// agents with their cell scratch, and the layout staging buffer a host transfer
// allocates.
uint64_t estimate_device_bytes(const Context* c)
{
	if (!c->mesh_set || c->S == 0)
		return 0;
	const uint64_t w = c->wsize, S = c->S, V = c->V, A = c->A;
	const uint64_t row_len = c->n[0] * S, pitch = round_up(row_len, 32 / w), rows = c->n[1] * c->n[2];
	uint64_t b = rows * pitch * w;               // field
	b += V * S * w;                              // staging of pcg_get_field / pcg_set_field
	for (int a = 0; a < c->dims; a++)            // coefficient tables (full and compressed; FP32: with lo parts)
		b += (7 * c->n[a] * S + 96 * S + 64) * w;
	b += 3 * 256 + 2 * S * 8;                    // words, mass
	b += c->K * (8 + S * (w + 1)) + 12 * S * (w + 1);
	if (c->bulk_mode == PCG_BULK_UNIFORM)
		b += 3 * S * w;
	else if (c->bulk_mode == PCG_BULK_PER_VOXEL)
		b += 3 * rows * pitch * w;
	if (A)
		b += A * (c->dims * 8 + 6 * S * 8 + 8 + 1 + 8 + 5 + 16 + 2 * term_stride(S, w) * w) + V * 8;
	return b;
}

int readback_ready(Context* c, uint64_t ticket, bool* done)
{
	if (ticket >= c->rb_issued)
		return fail(PCG_ERR_INVALID, "no readback with this ticket was started");
	DeviceGuard g(c->device);
	const int j = (int)(ticket % 2);
	*done = true;
	if (!c->rb_pending[j])
		return PCG_OK;
	// the slot's event is this readback's or a later one's on the same copy stream
	const cudaError_t e = cudaEventQuery(c->rb_done[j]);
	if (e == cudaErrorNotReady)
	{
		*done = false;
		return PCG_OK;
	}
	if (e != cudaSuccess)
		return fail(PCG_ERR_CUDA, std::string("readback: ") + cudaGetErrorString(e));
	c->rb_pending[j] = false;
	return PCG_OK;
}

} // namespace pcg

using pcg::Context;
using pcg::fail;


#define CTX_CHECK(ctx)                                                                                       \
	do                                                                                                       \
	{                                                                                                        \
		if (!(ctx))                                                                                          \
			return fail(PCG_ERR_INVALID, "null context");                                                    \
	} while (0)

extern "C" {

const char* pcg_last_error(void) { return pcg::g_last_error.c_str(); }

int pcg_create(pcg_context** out, int precision, int device)
{
	if (!out)
		return fail(PCG_ERR_INVALID, "null output pointer");
	if (precision != PCG_FP32 && precision != PCG_FP64)
		return fail(PCG_ERR_INVALID, "precision must be PCG_FP32 or PCG_FP64");
	int ndev = 0;
	cudaError_t e = cudaGetDeviceCount(&ndev);
	if (e != cudaSuccess || ndev == 0)
	{
		cudaGetLastError();
		return fail(PCG_ERR_CUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
	}
	if (device < 0 || device >= ndev)
		return fail(PCG_ERR_INVALID, "device index out of range");
	pcg::DeviceGuard g(device);
	auto* c = new pcg_context();
	c->device = device;
	c->precision = precision;
	c->wsize = precision == PCG_FP32 ? 4 : 8;
	cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
	// the stream and the device words are created on first use (initialize), so
	// that a context being configured holds no device resources at all
	*out = c;
	return PCG_OK;
}

int pcg_destroy(pcg_context* c)
{
	if (!c)
		return PCG_OK;
	pcg::DeviceGuard g(c->device);
	if (c->stream)
		stream_wait(c);
	if (c->rb_stream)
		cudaStreamSynchronize(c->rb_stream);
	pcg::collect_timings(c);
	pcg::DeviceBuffer* all[] = { &c->field,		 &c->coef[0],	&c->coef[1],	&c->coef[2],	 &c->a_vox,
								 &c->err,		&c->flags,		 &c->mass,		&c->tickets,
								 &c->staging,	 &c->dir_offsets, &c->dir_values, &c->dir_conds, &c->face_values,
								 &c->face_conds, &c->bulk[0],	&c->bulk[1],	&c->bulk[2],	 &c->a_pos,
								 &c->a_sec,		 &c->a_sat,		&c->a_upt,		&c->a_net,		 &c->a_vol,
								 &c->a_active,	 &c->a_internal, &c->a_frac,	&c->a_foff,		 &c->a_terms,
								 &c->a_reduced,
								 &c->owner,		 &c->counts,	&c->a_role,		&c->a_shared,	 &c->rb_staging[0],
								 &c->rb_staging[1], &c->a_rank,	&c->a_sorted,	&c->a_writers,	 &c->xy_segs,
								 &c->xy_done };
	for (auto* b : all)
		pcg::dfree(*b);
	pcg::dfree(c->slab); // after the pieces carved from it
	for (cudaEvent_t e : c->event_pool)
		cudaEventDestroy(e);
	for (int j = 0; j < 2; j++)
	{
		if (c->rb_packed[j])
			cudaEventDestroy(c->rb_packed[j]);
		if (c->rb_done[j])
			cudaEventDestroy(c->rb_done[j]);
	}
	if (c->rb_stream)
		cudaStreamDestroy(c->rb_stream);
	if (c->own_stream)
		cudaStreamDestroy(c->own_stream);
	pcg::pinned_words_put(c->h_words);
	if (c->ev_block)
		cudaEventDestroy(c->ev_block);
	delete c;
	return PCG_OK;
}

int pcg_set_stream(pcg_context* c, void* stream)
{
	CTX_CHECK(c);
	c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream; // may be created later
	return PCG_OK;
}

int pcg_get_stream(pcg_context* c, void** stream)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	const int rc = pcg::ensure_device_state(c);
	if (rc)
		return rc;
	*stream = c->stream;
	return PCG_OK;
}

int pcg_set_mesh(pcg_context* c, int dims, const int64_t bbmin[3], const int64_t bbmax[3], const uint64_t voxel[3])
{
	CTX_CHECK(c);
	c->generation++;
	if (c->initialized)
		return fail(PCG_ERR_INVALID, "the mesh cannot change after initialize");
	if (dims < 1 || dims > 3)
		return fail(PCG_ERR_INVALID, "dims must be 1, 2 or 3");
	uint64_t n[3] = { 1, 1, 1 };
	for (int a = 0; a < 3; a++)
		if (a < dims)
		{
			if (voxel[a] == 0)
				return fail(PCG_ERR_INVALID, "voxel shape must be positive on every mesh axis");
			if (bbmax[a] <= bbmin[a])
				return fail(PCG_ERR_INVALID, "bounding box max must exceed min on every mesh axis");
			n[a] = (uint64_t)((bbmax[a] - bbmin[a] + (int64_t)voxel[a] - 1) / (int64_t)voxel[a]); // mesh.cpp:16-27
		}
	for (int a = 0; a < 3; a++)
	{
		c->bbmin[a] = bbmin[a];
		c->bbmax[a] = bbmax[a];
		c->voxel[a] = voxel[a];
		c->n[a] = n[a];
	}
	c->dims = dims;
	c->mesh_set = true;
	c->V = n[0] * n[1] * n[2];
	if (c->V >= 0xffffffffull)
		return fail(PCG_ERR_UNSUPPORTED, "meshes beyond 2^32-1 voxels are not supported");
	return PCG_OK;
}

int pcg_get_grid(pcg_context* c, uint64_t grid[3])
{
	CTX_CHECK(c);
	for (int a = 0; a < 3; a++)
		grid[a] = c->n[a];
	return PCG_OK;
}

int pcg_set_substrates(pcg_context* c, uint64_t S, double dt, const double* D, const double* decay,
					   const double* initial)
{
	CTX_CHECK(c);
	c->generation++;
	if (c->initialized)
		return fail(PCG_ERR_INVALID, "substrates cannot change after initialize");
	if (S == 0 || !D || !decay || !initial)
		return fail(PCG_ERR_INVALID, "at least one substrate with D, decay and initial values is required");
	c->S = S;
	c->dt = dt;
	c->D.assign(D, D + S);
	c->decay.assign(decay, decay + S);
	c->init.assign(initial, initial + S);
	return PCG_OK;
}

int pcg_set_dirichlet_interior(pcg_context* c, uint64_t K, const uint64_t* voxels, const double* values,
							   const uint8_t* conditions)
{
	CTX_CHECK(c);
	c->generation++;
	if (!c->mesh_set || c->S == 0)
		return fail(PCG_ERR_INVALID, "mesh and substrates must be set before Dirichlet nodes");
	if (K && (!voxels || !values || !conditions))
		return fail(PCG_ERR_INVALID, "null Dirichlet arrays");
	for (uint64_t k = 0; k < K; k++)
		for (int d = 0; d < c->dims; d++)
			if (voxels[k * c->dims + d] >= c->n[d])
				return fail(PCG_ERR_INVALID, "Dirichlet node " + std::to_string(k) + " lies outside the mesh");
	pcg::DeviceGuard g(c->device);
	c->K = K;
	c->h_dir_voxels.assign(voxels, voxels + K * c->dims);
	c->h_dir_values.assign(values, values + K * c->S);
	c->h_dir_conds.assign(conditions, conditions + K * c->S);
	if (c->initialized)
		return c->wsize == 4 ? pcg::upload_dirichlet<float>(c) : pcg::upload_dirichlet<double>(c);
	return PCG_OK;
}

int pcg_set_dirichlet_boundary(pcg_context* c, int axis, int side, const double* values, const uint8_t* conditions)
{
	CTX_CHECK(c);
	c->generation++;
	if (axis < 0 || axis > 2 || side < 0 || side > 1)
		return fail(PCG_ERR_INVALID, "axis must be 0..2 and side 0 (min) or 1 (max)");
	if (c->S == 0)
		return fail(PCG_ERR_INVALID, "substrates must be set before boundary conditions");
	if (values && !conditions)
		return fail(PCG_ERR_INVALID, "boundary values need conditions");
	pcg::DeviceGuard g(c->device);
	c->face_on[axis][side] = values != nullptr;
	if (values)
	{
		c->h_face_values[axis][side].assign(values, values + c->S);
		c->h_face_conds[axis][side].assign(conditions, conditions + c->S);
	}
	if (c->initialized)
		return c->wsize == 4 ? pcg::upload_dirichlet<float>(c) : pcg::upload_dirichlet<double>(c);
	return PCG_OK;
}

int pcg_set_bulk(pcg_context* c, int mode, const double* supply, const double* uptake, const double* target)
{
	CTX_CHECK(c);
	c->generation++;
	if (mode != PCG_BULK_NONE && mode != PCG_BULK_UNIFORM && mode != PCG_BULK_PER_VOXEL)
		return fail(PCG_ERR_INVALID, "unknown bulk mode");
	if (mode != PCG_BULK_NONE && (!supply || !uptake || !target))
		return fail(PCG_ERR_INVALID, "bulk tables must not be null");
	if (mode != PCG_BULK_NONE && (!c->mesh_set || c->S == 0))
		return fail(PCG_ERR_INVALID, "mesh and substrates must be set before bulk tables");
	pcg::DeviceGuard g(c->device);
	c->bulk_mode = mode;
	const uint64_t cnt = mode == PCG_BULK_PER_VOXEL ? c->S * c->V : c->S;
	const double* src[3] = { supply, uptake, target };
	for (int k = 0; k < 3; k++)
	{
		if (mode == PCG_BULK_NONE)
			c->h_bulk[k].clear();
		else
			c->h_bulk[k].assign(src[k], src[k] + cnt);
	}
	if (c->initialized)
		return c->wsize == 4 ? pcg::upload_bulk<float>(c) : pcg::upload_bulk<double>(c);
	return PCG_OK;
}

int pcg_set_agents(pcg_context* c, uint64_t A, const double* positions, const double* secretion,
				   const double* saturation, const double* uptake, const double* net_export, const double* volumes,
				   const uint8_t* is_active, const double* internalized, const double* fraction_released,
				   int compute_internalized)
{
	CTX_CHECK(c);
	c->generation++;
	if (!c->mesh_set || c->S == 0)
		return fail(PCG_ERR_INVALID, "mesh and substrates must be set before agents");
	if (A >= 0xffffffffull)
		return fail(PCG_ERR_UNSUPPORTED, "at most 2^32-2 agents are supported");
	if (A && (!positions || !secretion || !saturation || !uptake || !net_export || !volumes || !is_active))
		return fail(PCG_ERR_INVALID, "null agent arrays");
	const uint64_t S = c->S, D = (uint64_t)c->dims;
	if (!c->initialized)
	{
		// staged on the host until initialize
		auto h = std::make_unique<Context::HostAgents>();
		h->pos.assign(positions, positions + A * D);
		h->sec.assign(secretion, secretion + A * S);
		h->sat.assign(saturation, saturation + A * S);
		h->upt.assign(uptake, uptake + A * S);
		h->net.assign(net_export, net_export + A * S);
		h->vol.assign(volumes, volumes + A);
		h->active.assign(is_active, is_active + A);
		if (internalized)
			h->internal.assign(internalized, internalized + A * S);
		if (fraction_released)
			h->frac.assign(fraction_released, fraction_released + A * S);
		c->staged_agents = std::move(h);
		c->A = A;
		c->compute_internalized = compute_internalized != 0;
		c->recompute_cells = true;
		return PCG_OK;
	}
	pcg::DeviceGuard g(c->device);
	return pcg::upload_agents(c, A, positions, secretion, saturation, uptake, net_export, volumes, is_active,
							  internalized, fraction_released, compute_internalized != 0);
}

int pcg_update_agents(pcg_context* c, const double* positions, const uint8_t* is_active)
{
	CTX_CHECK(c);
	if (c->A == 0)
		return PCG_OK;
	if (c->staged_agents)
	{
		if (positions)
			c->staged_agents->pos.assign(positions, positions + c->A * c->dims);
		if (is_active)
			c->staged_agents->active.assign(is_active, is_active + c->A);
		return PCG_OK;
	}
	pcg::DeviceGuard g(c->device);
	if (positions)
		PCG_CUDA_TRY(cudaMemcpyAsync(c->a_pos.ptr, positions, c->A * c->dims * sizeof(double),
									 cudaMemcpyHostToDevice, c->stream));
	if (is_active)
		PCG_CUDA_TRY(cudaMemcpyAsync(c->a_active.ptr, is_active, c->A, cudaMemcpyHostToDevice, c->stream));
	PCG_CUDA_TRY(stream_wait(c));
	return PCG_OK;
}

int pcg_set_internalized(pcg_context* c, const double* internalized)
{
	CTX_CHECK(c);
	if (c->A == 0)
		return PCG_OK;
	if (c->staged_agents)
	{
		c->staged_agents->internal.assign(internalized, internalized + c->A * c->S);
		return PCG_OK;
	}
	pcg::DeviceGuard g(c->device);
	std::vector<double> pairs;
	if (c->wsize == 4)
	{
		pcg::to_pairs(internalized, pairs, c->A * c->S);
		internalized = pairs.data();
	}
	PCG_CUDA_TRY(cudaMemcpyAsync(c->a_internal.ptr, internalized, c->A * c->S * sizeof(double),
								 cudaMemcpyHostToDevice, c->stream));
	PCG_CUDA_TRY(stream_wait(c));
	return PCG_OK;
}

int pcg_estimate_device_bytes(pcg_context* c, uint64_t* bytes)
{
	CTX_CHECK(c);
	if (!bytes)
		return fail(PCG_ERR_INVALID, "null argument");
	*bytes = pcg::estimate_device_bytes(c);
	return PCG_OK;
}

int pcg_initialize(pcg_context* c)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	return pcg::do_initialize(c);
}

int pcg_run_phases(pcg_context* c, uint32_t phases, int recompute_cells)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	int rc = pcg::do_initialize(c);
	if (rc)
		return rc;
	return pcg::run_phases(c, phases, recompute_cells != 0);
}

int pcg_solve(pcg_context* c, uint64_t iterations)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	int rc = pcg::do_initialize(c);
	if (rc)
		return rc;
	for (uint64_t it = 0; it < iterations; it++)
		if ((rc = pcg::run_phases(c, PCG_PHASE_ALL, c->recompute_cells)))
			return rc;
	c->recompute_cells = false;
	return PCG_OK;
}

int pcg_recompute_positional_data(pcg_context* c)
{
	CTX_CHECK(c);
	c->recompute_cells = true;
	return PCG_OK;
}

int pcg_release_internalized(pcg_context* c, uint64_t agent)
{
	CTX_CHECK(c);
	if (!c->compute_internalized)
		return PCG_OK; // cell_solver.cpp:353-354
	if (agent >= c->A)
		return fail(PCG_ERR_INVALID, "agent index out of range");
	pcg::DeviceGuard g(c->device);
	int rc = pcg::do_initialize(c);
	if (rc)
		return rc;
	return pcg::launch_release(c, agent);
}

// The device address of a host buffer mapped into the device's address space
// (memory from cudaHostAlloc, or registered with cudaHostRegister: pinned), else
// null (pageable memory).
static void* mapped_host_pointer(const void* host)
{
	cudaPointerAttributes at {};
	if (cudaPointerGetAttributes(&at, host) != cudaSuccess)
	{
		cudaGetLastError();
		return nullptr;
	}
	return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

int pcg_get_field(pcg_context* c, void* host, int layout, int dtype)
{
	CTX_CHECK(c);
	if (!host)
		return fail(PCG_ERR_INVALID, "null host buffer");
	if ((layout != PCG_LAYOUT_INTERLEAVED && layout != PCG_LAYOUT_PLANAR) ||
		(dtype != PCG_DTYPE_F32 && dtype != PCG_DTYPE_F64))
		return fail(PCG_ERR_INVALID, "bad layout or dtype");
	pcg::DeviceGuard g(c->device);
	int rc = pcg::do_initialize(c);
	if (rc)
		return rc;
	// Conversion on the device into a staging buffer, then one copy by the copy
	// engine.  (A kernel writing mapped host memory directly saves the staging pass,
	// about 6 % at the host link's rate, but holds SMs for the whole transfer,
	// which stalls other work on the device: a server's batched steps.)
	const size_t hw = dtype == PCG_DTYPE_F32 ? 4 : 8;
	if (layout == PCG_LAYOUT_INTERLEAVED && hw == c->wsize)
	{
		// the device rows are the host rows plus padding: one strided copy, no
		// kernel; queued once the stream is idle (see check_device)
		PCG_CUDA_TRY(stream_wait(c));
		PCG_CUDA_TRY(cudaMemcpy2DAsync(host, c->row_len * hw, c->field.ptr, c->pitch * hw, c->row_len * hw, c->rows,
									   cudaMemcpyDeviceToHost, c->stream));
		return pcg::check_device(c);
	}
	const size_t bytes = c->V * c->S * hw;
	if ((rc = pcg::dalloc(c, c->staging, bytes)))
		return rc;
	if ((rc = pcg::launch_to_host_layout(c, c->staging.ptr, layout, dtype)))
		return rc;
	// the copy is queued once the conversion is done (see check_device)
	PCG_CUDA_TRY(stream_wait(c));
	PCG_CUDA_TRY(cudaMemcpyAsync(host, c->staging.ptr, bytes, cudaMemcpyDeviceToHost, c->stream));
	return pcg::check_device(c);
}

int pcg_get_field_async(pcg_context* c, void* host, int layout, int dtype, uint64_t* ticket)
{
	CTX_CHECK(c);
	if (!host || !ticket)
		return fail(PCG_ERR_INVALID, "null host buffer or ticket");
	if ((layout != PCG_LAYOUT_INTERLEAVED && layout != PCG_LAYOUT_PLANAR) ||
		(dtype != PCG_DTYPE_F32 && dtype != PCG_DTYPE_F64))
		return fail(PCG_ERR_INVALID, "bad layout or dtype");
	pcg::DeviceGuard g(c->device);
	int rc = pcg::do_initialize(c);
	if (rc)
		return rc;
	if (!mapped_host_pointer(host))
	{
		// pageable memory: a copy to it would block anyway
		*ticket = c->rb_issued++;
		return pcg_get_field(c, host, layout, dtype);
	}
	if (!c->rb_stream)
	{
		PCG_CUDA_TRY(cudaStreamCreateWithFlags(&c->rb_stream, cudaStreamNonBlocking));
		for (int j = 0; j < 2; j++)
		{
			PCG_CUDA_TRY(cudaEventCreateWithFlags(&c->rb_packed[j], cudaEventDisableTiming));
			PCG_CUDA_TRY(cudaEventCreateWithFlags(&c->rb_done[j], cudaEventDisableTiming));
		}
	}
	const int j = (int)(c->rb_issued % 2);
	const size_t bytes = c->V * c->S * (dtype == PCG_DTYPE_F32 ? 4 : 8);
	if (c->rb_staging[j].bytes < bytes)
	{
		if (c->rb_pending[j])
			PCG_CUDA_TRY(cudaEventSynchronize(c->rb_done[j])); // its last copy still reads it
		if ((rc = pcg::dalloc(c, c->rb_staging[j], bytes)))
			return rc;
	}
	// the slot's previous copy to the host must have read the buffer before it is
	// overwritten; the main stream waits for it on the device, not the host
	if (c->rb_pending[j])
		PCG_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->rb_done[j], 0));
	if ((rc = pcg::launch_to_host_layout(c, c->rb_staging[j].ptr, layout, dtype)))
		return rc;
	PCG_CUDA_TRY(cudaEventRecord(c->rb_packed[j], c->stream));
	PCG_CUDA_TRY(cudaStreamWaitEvent(c->rb_stream, c->rb_packed[j], 0));
	PCG_CUDA_TRY(cudaMemcpyAsync(host, c->rb_staging[j].ptr, bytes, cudaMemcpyDeviceToHost, c->rb_stream));
	PCG_CUDA_TRY(cudaEventRecord(c->rb_done[j], c->rb_stream));
	c->rb_pending[j] = true;
	*ticket = c->rb_issued++;
	return PCG_OK;
}

int pcg_wait_field(pcg_context* c, uint64_t ticket)
{
	CTX_CHECK(c);
	if (ticket >= c->rb_issued)
		return fail(PCG_ERR_INVALID, "no readback with this ticket was started");
	pcg::DeviceGuard g(c->device);
	const int j = (int)(ticket % 2);
	// the slot's event belongs to this readback or to a later one in the same
	// copy stream, which completes after it: either way the slot is idle after it
	if (c->rb_pending[j])
	{
		cudaError_t e = cudaEventSynchronize(c->rb_done[j]);
		if (e != cudaSuccess)
			return fail(PCG_ERR_CUDA, std::string("readback: ") + cudaGetErrorString(e));
		c->rb_pending[j] = false;
	}
	// no device error-word read here: a copy from the device would queue behind the
	// readbacks still running and wait for them; kernel errors surface at the next
	// call that synchronises the context's stream
	return PCG_OK;
}

int pcg_set_field(pcg_context* c, const void* host, int layout, int dtype)
{
	CTX_CHECK(c);
	if (!host)
		return fail(PCG_ERR_INVALID, "null host buffer");
	if ((layout != PCG_LAYOUT_INTERLEAVED && layout != PCG_LAYOUT_PLANAR) ||
		(dtype != PCG_DTYPE_F32 && dtype != PCG_DTYPE_F64))
		return fail(PCG_ERR_INVALID, "bad layout or dtype");
	pcg::DeviceGuard g(c->device);
	int rc = pcg::do_initialize(c);
	if (rc)
		return rc;
	const size_t hw = dtype == PCG_DTYPE_F32 ? 4 : 8;
	if (layout == PCG_LAYOUT_INTERLEAVED && hw == c->wsize)
	{
		PCG_CUDA_TRY(cudaMemcpy2DAsync(c->field.ptr, c->pitch * hw, host, c->row_len * hw, c->row_len * hw, c->rows,
									   cudaMemcpyHostToDevice, c->stream));
		return pcg::check_device(c);
	}
	const size_t bytes = c->V * c->S * hw;
	if ((rc = pcg::dalloc(c, c->staging, bytes)))
		return rc;
	PCG_CUDA_TRY(cudaMemcpyAsync(c->staging.ptr, host, bytes, cudaMemcpyHostToDevice, c->stream));
	if ((rc = pcg::launch_from_host_layout(c, c->staging.ptr, layout, dtype)))
		return rc;
	return pcg::check_device(c);
}

int pcg_get_density(pcg_context* c, uint64_t s, uint64_t x, uint64_t y, uint64_t z, double* value)
{
	CTX_CHECK(c);
	if (!c->initialized)
		return fail(PCG_ERR_INVALID, "not initialized");
	if (s >= c->S || x >= c->n[0] || y >= c->n[1] || z >= c->n[2])
		return fail(PCG_ERR_INVALID, "density index out of range");
	pcg::DeviceGuard g(c->device);
	int rc = pcg::check_device(c);
	if (rc)
		return rc;
	const uint64_t off = (z * c->n[1] + y) * c->pitch + x * c->S + s;
	if (c->wsize == 4)
	{
		float v;
		PCG_CUDA_TRY(cudaMemcpy(&v, static_cast<float*>(c->field.ptr) + off, 4, cudaMemcpyDeviceToHost));
		*value = v;
	}
	else
		PCG_CUDA_TRY(cudaMemcpy(value, static_cast<double*>(c->field.ptr) + off, 8, cudaMemcpyDeviceToHost));
	return PCG_OK;
}

int pcg_get_internalized(pcg_context* c, double* host)
{
	CTX_CHECK(c);
	if (c->staged_agents)
	{
		const std::vector<double>& I = c->staged_agents->internal;
		if (I.empty())
			std::fill(host, host + c->A * c->S, 0.0);
		else
			std::copy(I.begin(), I.end(), host);
		return PCG_OK;
	}
	pcg::DeviceGuard g(c->device);
	int rc = pcg::check_device(c);
	if (rc)
		return rc;
	if (c->A)
	{
		PCG_CUDA_TRY(cudaMemcpy(host, c->a_internal.ptr, c->A * c->S * sizeof(double), cudaMemcpyDeviceToHost));
		if (c->wsize == 4)
			pcg::from_pairs(host, c->A * c->S);
	}
	return PCG_OK;
}

int pcg_get_counts(pcg_context* c, uint32_t* host)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	int rc = pcg::check_device(c);
	if (rc)
		return rc;
	if (!c->counts.ptr)
	{
		memset(host, 0, c->V * sizeof(uint32_t));
		return PCG_OK;
	}
	PCG_CUDA_TRY(cudaMemcpy(host, c->counts.ptr, c->V * sizeof(uint32_t), cudaMemcpyDeviceToHost));
	return PCG_OK;
}

int pcg_get_conflict(pcg_context* c, int* conflict)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	int rc = pcg::check_device(c);
	if (rc)
		return rc;
	uint32_t f = 0;
	PCG_CUDA_TRY(cudaMemcpy(&f, c->flags.ptr, sizeof(f), cudaMemcpyDeviceToHost));
	*conflict = f != 0;
	return PCG_OK;
}

int pcg_mass(pcg_context* c, double* host)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	int rc = pcg::do_initialize(c);
	if (rc)
		return rc;
	if ((rc = pcg::launch_mass(c, static_cast<double*>(c->mass.ptr))))
		return rc;
	PCG_CUDA_TRY(cudaMemcpyAsync(host, c->mass.ptr, c->S * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
	return pcg::check_device(c);
}

// Buffers of the mass check and its per-substrate sweep factors: each sweep
// matrix has column sums 1 + decay*dt/dims, plus r = dt*D/h^2 on an axis of
// length 1, whose single diagonal entry has r subtracted once rather than twice
// (diffusion_solver.cpp:29-86), so the sweeps divide every substrate's total by
// the product of those sums over the mesh's axes.
static int prepare_mass_check(Context* c)
{
	int rc;
	if ((rc = pcg::dalloc(c, c->mc_tot, 2 * c->S * sizeof(double))) ||
		(rc = pcg::dalloc(c, c->mc_out, 4 * c->S * sizeof(double))))
		return rc;
	PCG_CUDA_TRY(cudaMemsetAsync(c->mc_tot.ptr, 0, 2 * c->S * sizeof(double), c->stream));
	std::vector<double> h(4 * c->S, 0.0);
	for (uint64_t s = 0; s < c->S; s++)
	{
		double p = 1.0;
		for (int a = 0; a < c->dims; a++)
		{
			const double h = (double)c->voxel[a];
			const double r = c->n[a] == 1 ? c->dt * c->D[s] / (h * h) : 0.0;
			p *= 1.0 + c->decay[s] * c->dt / (double)c->dims + r;
		}
		h[3 * c->S + s] = p;
	}
	PCG_CUDA_TRY(pcg::stream_wait(c));
	PCG_CUDA_TRY(cudaMemcpyAsync(c->mc_out.ptr, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
	PCG_CUDA_TRY(pcg::stream_wait(c));
	c->mass_checked_steps = 0;
	return PCG_OK;
}

int pcg_set_sweep_fusion(pcg_context* c, int enable, uint64_t slab_bytes, uint32_t lag)
{
	CTX_CHECK(c);
	c->fuse_xy = enable != 0;
	if (slab_bytes)
		c->xy_slab_bytes = slab_bytes;
	if (lag)
		c->xy_lag = lag;
	return PCG_OK;
}

int pcg_set_mass_check(pcg_context* c, int enable)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	int rc = pcg::do_initialize(c);
	if (rc)
		return rc;
	if (enable && (rc = prepare_mass_check(c)))
		return rc;
	if (c->mass_check != (enable != 0))
		c->generation++; // a batch holding this context rebuilds its descriptors
	c->mass_check = enable != 0;
	return PCG_OK;
}

int pcg_get_mass_check(pcg_context* c, double* mass_before, double* mass_after, double* worst_residual,
					   uint64_t* steps_checked)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	if (!c->mc_out.ptr)
		return fail(PCG_ERR_INVALID, "the mass check was never enabled");
	std::vector<double> h(3 * c->S);
	PCG_CUDA_TRY(pcg::stream_wait(c));
	PCG_CUDA_TRY(cudaMemcpyAsync(h.data(), c->mc_out.ptr, h.size() * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
	const int rc = pcg::check_device(c);
	if (rc)
		return rc;
	for (uint64_t s = 0; s < c->S; s++)
	{
		if (mass_before)
			mass_before[s] = h[s];
		if (mass_after)
			mass_after[s] = h[c->S + s];
		if (worst_residual)
			worst_residual[s] = h[2 * c->S + s];
	}
	if (steps_checked)
		*steps_checked = c->mass_checked_steps;
	return PCG_OK;
}

int pcg_synchronize(pcg_context* c)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	return pcg::check_device(c);
}

int pcg_get_field_device(pcg_context* c, void** ptr, uint64_t* elem_bytes, uint64_t* pitch)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	int rc = pcg::do_initialize(c);
	if (rc)
		return rc;
	*ptr = c->field.ptr;
	*elem_bytes = c->wsize;
	*pitch = c->pitch;
	return PCG_OK;
}

int pcg_get_agents_device(pcg_context* c, double** positions, uint8_t** is_active)
{
	CTX_CHECK(c);
	if (!positions || !is_active)
		return fail(PCG_ERR_INVALID, "null argument");
	pcg::DeviceGuard g(c->device);
	int rc = pcg::do_initialize(c);
	if (rc)
		return rc;
	if (c->A == 0)
		return fail(PCG_ERR_INVALID, "the context holds no agents");
	*positions = static_cast<double*>(c->a_pos.ptr);
	*is_active = static_cast<uint8_t*>(c->a_active.ptr);
	return PCG_OK;
}

int pcg_set_kernel_timing(pcg_context* c, int enable)
{
	CTX_CHECK(c);
	c->timing = enable != 0;
	// The cell kernels' bytes scale with device-side counts (agents of shared
	// voxels, agents that write a voxel), copied to pinned words after every timed
	// ballot.  A ballot built before timing was enabled leaves them here.
	if (c->timing && c->initialized && c->A && c->ballot_kind == 1 && c->flags.ptr)
	{
		pcg::DeviceGuard g(c->device);
		if (!c->h_words && !(c->h_words = pcg::pinned_words_get()))
			return fail(PCG_ERR_NOMEM, "pinned host memory for the device words");
		PCG_CUDA_TRY(stream_wait(c));
		PCG_CUDA_TRY(cudaMemcpy(c->h_words + 2, static_cast<uint32_t*>(c->flags.ptr) + 2, sizeof(uint32_t),
								cudaMemcpyDeviceToHost));
		PCG_CUDA_TRY(cudaMemcpy(c->h_words + 3, static_cast<uint32_t*>(c->flags.ptr) + 4, sizeof(uint32_t),
								cudaMemcpyDeviceToHost));
		c->shared_agents = c->h_words[2];
		c->writer_agents = c->h_words[3];
	}
	return PCG_OK;
}

int pcg_get_kernel_stats(pcg_context* c, pcg_kernel_stat* stats, uint64_t cap, uint64_t* count)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	stream_wait(c);
	pcg::collect_timings(c);
	*count = pcg::K_COUNT;
	for (uint64_t k = 0; k < cap && k < (uint64_t)pcg::K_COUNT; k++)
	{
		memset(&stats[k], 0, sizeof(pcg_kernel_stat));
		snprintf(stats[k].name, sizeof(stats[k].name), "%s", pcg::kernel_name((int)k));
		stats[k].launches = c->stats[k].launches;
		stats[k].total_ms = c->stats[k].total_ms;
		stats[k].algorithmic_bytes = c->stats[k].bytes;
	}
	return PCG_OK;
}

int pcg_reset_kernel_stats(pcg_context* c)
{
	CTX_CHECK(c);
	pcg::DeviceGuard g(c->device);
	stream_wait(c);
	pcg::collect_timings(c);
	for (auto& s : c->stats)
		s = pcg::KernelStat {};
	c->launches = 0;
	return PCG_OK;
}

int pcg_get_launch_count(pcg_context* c, uint64_t* launches)
{
	CTX_CHECK(c);
	*launches = c->launches;
	return PCG_OK;
}

} // extern "C"
