// field_device.cuh -- per-item device code of the Dirichlet and bulk phases,
// shared by the single-domain kernels (field_ops.cu) and the batched ones (batch.cu).
//
// Dirichlet (openmp_solver/src/dirichlet_solver.cpp:22-93): the reference writes
// the x-min, x-max, y-min, y-max, z-min, z-max faces one after another (a later
// face wins on shared edges) and then the interior voxels.  A face item is one
// (face voxel, substrate); it applies the face of highest precedence whose
// condition holds, so edges resolve exactly as the sequential order does.
//
// Bulk (openmp_solver/src/bulk_solver.cpp:12-49): D = (D + dt*S*T)/(1 + dt*(U+S)).
#pragma once

#include "pcg_internal.cuh"

namespace pcg {

struct FaceArgs
{
	void* field;
	const void* values; // real [6*S]: face f = axis*2 + side
	const uint8_t* conds;
	uint32_t face_mask; // bit f set when face f exists
	uint64_t S, nx, ny, nz, pitch;
	uint64_t cnt_x, cnt_y, cnt_z; // voxels on each pair of faces
	uint64_t total;               // face voxels (all pairs)
};

// Fills the face geometry of a mesh from its per-face presence.
inline FaceArgs make_face_args(const Context* c)
{
	FaceArgs a {};
	uint32_t mask = 0;
	for (int axis = 0; axis < c->dims; axis++)
		for (int side = 0; side < 2; side++)
			if (c->face_on[axis][side])
				mask |= 1u << (axis * 2 + side);
	const uint64_t nx = c->n[0], ny = c->n[1], nz = c->n[2];
	a.field = c->field.ptr;
	a.values = c->face_values.ptr;
	a.conds = static_cast<const uint8_t*>(c->face_conds.ptr);
	a.face_mask = mask;
	a.S = c->S;
	a.nx = nx, a.ny = ny, a.nz = nz;
	a.pitch = c->pitch;
	a.cnt_x = (mask & 0x3) ? 2 * ny * nz : 0;
	a.cnt_y = (mask & 0xc) ? 2 * nx * nz : 0;
	a.cnt_z = (mask & 0x30) ? 2 * nx * ny : 0;
	a.total = a.cnt_x + a.cnt_y + a.cnt_z;
	return a;
}

#ifdef __CUDACC__
namespace fielddev {

// Face item idx < total*S.
template <typename T>
__device__ __forceinline__ void face_item(const FaceArgs& a, uint64_t idx)
{
	const T* vals = static_cast<const T*>(a.values);
	T* f = static_cast<T*>(a.field);
	const uint64_t s = idx % a.S;
	uint64_t k = idx / a.S;
	uint64_t x, y, z;
	if (k < a.cnt_x)
	{ // x faces: k -> (side, y, z)
		const uint64_t per = a.ny * a.nz;
		x = (k / per) ? a.nx - 1 : 0;
		y = (k % per) % a.ny;
		z = (k % per) / a.ny;
	}
	else if ((k -= a.cnt_x) < a.cnt_y)
	{
		const uint64_t per = a.nx * a.nz;
		y = (k / per) ? a.ny - 1 : 0;
		x = (k % per) % a.nx;
		z = (k % per) / a.nx;
	}
	else
	{
		k -= a.cnt_y;
		const uint64_t per = a.nx * a.ny;
		z = (k / per) ? a.nz - 1 : 0;
		x = (k % per) % a.nx;
		y = (k % per) / a.nx;
	}
	// precedence: the reference applies faces 0..5 in order, so scan 5..0
	const uint64_t coord[3] = { x, y, z };
	const uint64_t last[3] = { a.nx - 1, a.ny - 1, a.nz - 1 };
	for (int fi = 5; fi >= 0; fi--)
	{
		if (!(a.face_mask & (1u << fi)))
			continue;
		const int axis = fi >> 1, side = fi & 1;
		if (coord[axis] != (side ? last[axis] : 0))
			continue;
		if (a.conds[fi * a.S + s])
		{
			f[(z * a.ny + y) * a.pitch + x * a.S + s] = vals[fi * a.S + s];
			break;
		}
	}
}

// One row of the bulk update by the 32 lanes of a warp; a lane walks the row's
// (x,s) run with its substrate index advanced incrementally.
template <typename T, bool PER_VOXEL>
__device__ __forceinline__ void bulk_row(T* field, const T* supply, const T* uptake, const T* target,
										 uint64_t row_len, uint64_t pitch, uint64_t r, uint32_t S, T dt, int lane)
{
	const uint32_t s_step = 32 % S;
	T* row = field + r * pitch;
	uint32_t s = (uint32_t)lane % S;
	for (uint64_t k = lane; k < row_len; k += 32)
	{
		T Sr, U, Tt;
		if (PER_VOXEL)
		{
			const uint64_t o = r * pitch + k;
			Sr = supply[o];
			U = uptake[o];
			Tt = target[o];
		}
		else
		{
			Sr = supply[s];
			U = uptake[s];
			Tt = target[s];
		}
		// bulk_solver.cpp:12-49: D' = (D + dt S T) / (1 + dt (U + S)); FP32 as
		// D + (dt S T - D dt (U + S)) / (1 + dt (U + S)), so that a small dt (U + S)
		// keeps its precision (its sum with 1 only scales the correction)
		if constexpr (sizeof(T) == 4)
		{
			const T a = dt * Sr * Tt, b = dt * (U + Sr);
			row[k] = row[k] + fmaf(-row[k], b, a) / (T(1) + b);
		}
		else
			row[k] = (row[k] + dt * Sr * Tt) / (T(1) + dt * (U + Sr));
		s += s_step;
		if (s >= S)
			s -= S;
	}
}

// The boundary faces of the voxels of one solved y/z column in shared memory (the
// last sweep of the step, so these are the values the reference's Dirichlet pass
// would write next).  The column is element c = x*S + s of a row at all n points
// of the swept axis (stride `stride`); `o` is the index along the third axis.
// Faces apply in the reference's order x-min, x-max, y-min, y-max, z-min, z-max,
// a later face winning: first the faces whose plane holds the whole column, then
// the two faces of the swept axis at its ends.
template <typename T, int AXIS>
__device__ __forceinline__ void faces_on_column(const FaceArgs& f, T* col, uint32_t n, uint32_t stride, uint64_t c,
												uint64_t o)
{
	if (!f.face_mask || c >= f.nx * f.S)
		return;
	const T* vals = static_cast<const T*>(f.values);
	const uint32_t s = (uint32_t)(c % f.S);
	const uint64_t x = c / f.S;
	bool has = false;
	T v = T(0);
	auto take = [&](int fi) {
		if (((f.face_mask >> fi) & 1u) && f.conds[fi * f.S + s])
		{
			v = vals[fi * f.S + s];
			has = true;
		}
	};
	if (x == 0)
		take(0);
	if (x == f.nx - 1)
		take(1);
	const uint64_t n_other = AXIS == 2 ? f.ny : f.nz; // the axis that is neither x nor swept
	const int f_other = AXIS == 2 ? 2 : 4;
	if (o == 0)
		take(f_other);
	if (o == n_other - 1)
		take(f_other + 1);
	if (has)
		for (uint32_t j = 0; j < n; j++)
			col[(uint64_t)j * stride] = v;
	const int f_swept = AXIS == 2 ? 4 : 2;
	if (((f.face_mask >> f_swept) & 1u) && f.conds[f_swept * f.S + s])
		col[0] = vals[f_swept * f.S + s];
	if (((f.face_mask >> (f_swept + 1)) & 1u) && f.conds[(f_swept + 1) * f.S + s])
		col[(uint64_t)(n - 1) * stride] = vals[(f_swept + 1) * f.S + s];
}

} // namespace fielddev
#endif

} // namespace pcg
