// noalloc.cu -- the cell secretion/uptake step without any device allocation.
//
// Some callers cannot let a library allocate device memory: simulation frameworks
// that hand out all GPU memory from their own fixed pool or arena (a cudaMalloc
// behind their back breaks their budget and accounting), and loops that must not
// take the implicit device synchronisation of cudaMalloc/cudaFree.  For them,
// pcg_cells_noalloc runs the cell step on buffers the caller already owns; the
// only extra memory it needs -- ballot slots, per-voxel counts and per-agent
// reduced terms -- lives in one file-scope __device__ array of a fixed size that
// every GPU loading this library holds until the process exits.
#include <mutex>

#include "pcg_internal.cuh"

namespace {

// 16 MiB of scratch: 8 bytes per voxel (group start + count) plus 25 + 24*S bytes
// per agent (voxel index, field offset, shared-voxel list entry, rank in the voxel,
// grouped (agent, voxel) slot, ballot role, six FP32 terms per substrate).
constexpr size_t kScratchBytes = size_t(16) << 20;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
void* g_scratch_addr[kMaxDevices] = {}; // device address of g_scratch, per device

// The host-side symbol g_scratch is only a stand-in; kernels need the device
// address, looked up once per device with that device current.
int scratch_address(int device, unsigned char** out)
{
	if (device < 0 || device >= kMaxDevices)
		return pcg::fail(PCG_ERR_UNSUPPORTED, "device index beyond the scratch table");
	std::lock_guard<std::mutex> lock(g_mutex);
	if (!g_scratch_addr[device])
	{
		void* p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
		if (e != cudaSuccess)
			return pcg::fail(PCG_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
		g_scratch_addr[device] = p;
	}
	*out = static_cast<unsigned char*>(g_scratch_addr[device]);
	return PCG_OK;
}

size_t align256(size_t v) { return (v + 255) / 256 * 256; }

} // namespace

extern "C" int pcg_cells_noalloc(float* field, uint64_t pitch, int dims, const int64_t bbox_min[3],
								 const uint64_t voxel_shape[3], const uint64_t grid_shape[3], uint64_t substrates,
								 double dt, uint64_t agents, const double* positions, const double* secretion,
								 const double* saturation, const double* uptake, const double* net_export,
								 const double* volumes, const uint8_t* is_active, double* internalized,
								 int compute_internalized, void* stream)
{
	using pcg::fail;
	if (dims < 1 || dims > 3 || substrates == 0 || !bbox_min || !voxel_shape || !grid_shape)
		return fail(PCG_ERR_INVALID, "pcg_cells_noalloc: bad mesh or substrate count");
	if (!field)
		return fail(PCG_ERR_INVALID, "pcg_cells_noalloc: null field");
	uint64_t V = 1;
	for (int d = 0; d < 3; d++)
	{
		if (grid_shape[d] == 0 || (d < dims && voxel_shape[d] == 0))
			return fail(PCG_ERR_INVALID, "pcg_cells_noalloc: empty grid axis or zero voxel shape");
		if (d >= dims && grid_shape[d] != 1)
			return fail(PCG_ERR_INVALID, "pcg_cells_noalloc: grid_shape must be 1 on the axes beyond dims");
		if (__builtin_mul_overflow(V, grid_shape[d], &V))
			return fail(PCG_ERR_UNSUPPORTED, "pcg_cells_noalloc: the voxel count overflows 64 bits");
	}
	uint64_t row = 0, field_elems = 0, terms = 0;
	if (__builtin_mul_overflow(grid_shape[0], substrates, &row))
		return fail(PCG_ERR_UNSUPPORTED, "pcg_cells_noalloc: nx * substrates overflows 64 bits");
	if (pitch < row)
		return fail(PCG_ERR_INVALID, "pcg_cells_noalloc: pitch shorter than a row (nx * substrates)");
	// voxel indices, agent indices and field offsets are 32-bit on the device
	if (V >= 0xffffffffull)
		return fail(PCG_ERR_UNSUPPORTED, "pcg_cells_noalloc: meshes of 2^32 - 1 or more voxels are not supported");
	if (agents >= 0xffffffffull)
		return fail(PCG_ERR_UNSUPPORTED, "pcg_cells_noalloc: 2^32 - 1 or more agents are not supported");
	if (__builtin_mul_overflow(pitch, grid_shape[1] * grid_shape[2], &field_elems) || field_elems >= (1ull << 32))
		return fail(PCG_ERR_UNSUPPORTED,
					"pcg_cells_noalloc: fields of 2^32 or more elements (pitch * ny * nz) are not supported");
	if (__builtin_mul_overflow(agents, substrates, &terms) || __builtin_mul_overflow(terms, sizeof(float), &terms))
		return fail(PCG_ERR_UNSUPPORTED, "pcg_cells_noalloc: agents * substrates overflows 64 bits");
	if (agents && (!positions || !secretion || !saturation || !uptake || !net_export || !volumes || !is_active ||
				   (compute_internalized && !internalized)))
		return fail(PCG_ERR_INVALID, "pcg_cells_noalloc: null agent array");
	if (agents == 0)
		return PCG_OK;
	// every piece below is at most kScratchBytes before the total is compared
	if (V > kScratchBytes || terms > kScratchBytes)
		return fail(PCG_ERR_UNSUPPORTED,
					"pcg_cells_noalloc: the mesh and agents need more than the fixed " + std::to_string(kScratchBytes) +
						" bytes of scratch (about 8 bytes per voxel + (25 + 24*S) bytes per agent)");

	// scratch layout: flags | err | owner[V] | counts[V] | vox[A] | foff[A] | shared[A] | rank[A] | sorted[A] |
	// role[A] | 6 x terms[A*S]
	size_t off = 0;
	const size_t o_flags = off;
	off += 256;
	const size_t o_err = off;
	off += 256;
	const size_t o_owner = off;
	off = align256(off + V * 4);
	const size_t o_counts = off;
	off = align256(off + V * 4);
	const size_t o_vox = off;
	off = align256(off + agents * 4);
	const size_t o_foff = off;
	off = align256(off + agents * 4);
	const size_t o_shared = off;
	off = align256(off + agents * 4);
	const size_t o_rank = off;
	off = align256(off + agents * 4);
	const size_t o_sorted = off;
	off = align256(off + agents * 8);
	const size_t o_role = off;
	off = align256(off + agents);
	size_t o_terms[6];
	for (int k = 0; k < 6; k++)
	{
		o_terms[k] = off;
		off = align256(off + terms);
	}
	if (off > kScratchBytes)
		return fail(PCG_ERR_UNSUPPORTED,
					"pcg_cells_noalloc: the mesh and agents need " + std::to_string(off) +
						" bytes of scratch, more than the fixed " + std::to_string(kScratchBytes) +
						" (about 8 bytes per voxel + (25 + 24*S) bytes per agent)");

	int device = 0;
	cudaError_t e = cudaGetDevice(&device);
	if (e != cudaSuccess)
		return fail(PCG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
	unsigned char* base = nullptr;
	int rc = scratch_address(device, &base);
	if (rc)
		return rc;

	pcg::CellStepBuffers b {};
	b.dims = dims;
	b.A = agents;
	b.S = substrates;
	for (int d = 0; d < 3; d++)
	{
		b.n[d] = grid_shape[d];
		b.bbmin[d] = bbox_min[d];
		b.voxel[d] = voxel_shape[d];
	}
	b.pitch = pitch;
	b.dt = dt;
	b.pos = positions;
	b.sec = secretion;
	b.sat = saturation;
	b.upt = uptake;
	b.net = net_export;
	b.vol = volumes;
	b.active = is_active;
	b.internal = internalized;
	b.internalized = compute_internalized ? 1 : 0;
	b.field = field;
	b.flags = reinterpret_cast<uint32_t*>(base + o_flags);
	b.err = reinterpret_cast<uint32_t*>(base + o_err);
	b.owner = reinterpret_cast<uint32_t*>(base + o_owner);
	b.counts = reinterpret_cast<uint32_t*>(base + o_counts);
	b.vox = reinterpret_cast<uint32_t*>(base + o_vox);
	b.foff = reinterpret_cast<uint32_t*>(base + o_foff);
	b.shared = reinterpret_cast<uint32_t*>(base + o_shared);
	b.rank = reinterpret_cast<uint32_t*>(base + o_rank);
	b.sorted = reinterpret_cast<uint2*>(base + o_sorted);
	b.role = base + o_role;
	float** t[6] = { &b.num, &b.den, &b.fac, &b.rnum, &b.rden, &b.rfac };
	for (int k = 0; k < 6; k++)
		*t[k] = reinterpret_cast<float*>(base + o_terms[k]);

	cudaStream_t s = static_cast<cudaStream_t>(stream);
	// the array keeps the previous call's contents: the error word starts at zero
	e = cudaMemsetAsync(b.err, 0, sizeof(uint32_t), s);
	if (e != cudaSuccess)
		return fail(PCG_ERR_CUDA, std::string("cudaMemsetAsync(scratch): ") + cudaGetErrorString(e));
	if ((rc = pcg::launch_cells_fp32_buffers(b, s)))
		return rc;
	uint32_t word = 0;
	e = cudaMemcpyAsync(&word, b.err, sizeof(word), cudaMemcpyDeviceToHost, s);
	if (e == cudaSuccess)
		e = cudaStreamSynchronize(s);
	if (e != cudaSuccess)
		return fail(PCG_ERR_CUDA, std::string("pcg_cells_noalloc: ") + cudaGetErrorString(e));
	if (word & pcg::DEV_ERR_AGENT_OUTSIDE)
		return fail(PCG_ERR_DEVICE, "device fault: an active agent lies outside the mesh");
	return PCG_OK;
}
