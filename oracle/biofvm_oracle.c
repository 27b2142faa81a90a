/*
 * biofvm_oracle.c -- CPU restatement of the reference OpenMP BioFVM solver.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GB300 kernels and the timed CPU
 * baseline.  Nothing in the product path links it.
 *
 * Each function cites the reference file:line whose arithmetic it restates
 * (paths relative to reactions-diffusion/biofvm/).  The operation order of every
 * floating-point expression follows the reference source; the library is built
 * with -ffp-contract=off so x86 and Arm hosts give identical bits.
 *
 * Deliberate, documented differences from the reference:
 *  - y/z sweeps use the coefficients of each line's own substrate.  The reference
 *    OpenMP tiles (diffusion_solver.cpp:399-401, 415-447) index the replicated
 *    coefficient table by the position inside a 48-wide tile, which selects the
 *    right substrate only when S divides 48; for S in {1,2,3,4,6,8,12,16,24,48}
 *    the two agree exactly.  The Thrust backend (thrust diffusion_solver.cpp:
 *    167-195) and the formula in diffusion_solver.h:11-40 use per-substrate
 *    coefficients, as here.
 *  - Cell ballots are resolved serially in agent-index order, so the winner of a
 *    voxel is its lowest-index active agent and the reduced sums are added in
 *    agent-index order.  The reference resolves them with racing CAS/atomic adds
 *    (cell_solver.cpp:79-129); any winner gives the same densities up to the
 *    order of the floating-point sums.
 *  - An active agent whose voxel index falls outside the grid is an error here;
 *    the reference only asserts (mesh.cpp:39-44) and would index out of range.
 */
#include "biofvm_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define NO_BALLOT UINT64_MAX
#define XS_TILE 48

struct orc_state
{
	int dims;
	int64_t bbmin[3], bbmax[3];
	uint64_t voxel[3];
	uint64_t n[3];
	int mesh_set;
	int threads;

	uint64_t S;
	double dt;
	double *D, *decay, *init;

	uint64_t K;
	uint64_t* dir_voxels;
	double* dir_values;
	uint8_t* dir_conds;

	/* boundary: [axis][side] -> values/conds of length S, NULL when absent */
	double* bnd_values[3][2];
	uint8_t* bnd_conds[3][2];

	int bulk_mode;
	double *bulk_supply, *bulk_uptake, *bulk_target;

	uint64_t A;
	double *pos, *sec, *sat, *upt, *net, *vol, *internalized, *frac_rel;
	uint8_t* active;
	int compute_internalized;

	/* solver state */
	int initialized;
	int recompute_cells;
	double* field;
	double *b[3], *e[3], *c[3];
	double *num, *den, *fac, *rnum, *rden, *rfac;
	uint64_t* ballots;
	uint64_t* agent_voxel;
	int is_conflict;
};

static __thread char g_err[512];

static int fail(const char* fmt, ...)
{
	va_list ap;
	va_start(ap, fmt);
	vsnprintf(g_err, sizeof g_err, fmt, ap);
	va_end(ap);
	return -1;
}

const char* orc_last_error(void) { return g_err; }

static void* dup_array(const void* src, size_t bytes)
{
	if (!src || bytes == 0)
		return NULL;
	void* p = malloc(bytes);
	memcpy(p, src, bytes);
	return p;
}

orc_state* orc_create(void)
{
	orc_state* st = (orc_state*)calloc(1, sizeof(orc_state));
	st->recompute_cells = 1;
	st->threads = 0;
	return st;
}

static void free_solver(orc_state* st)
{
	free(st->field);
	st->field = NULL;
	for (int a = 0; a < 3; a++)
	{
		free(st->b[a]);
		free(st->e[a]);
		free(st->c[a]);
		st->b[a] = st->e[a] = st->c[a] = NULL;
	}
	free(st->num), free(st->den), free(st->fac);
	free(st->rnum), free(st->rden), free(st->rfac);
	free(st->ballots), free(st->agent_voxel);
	st->num = st->den = st->fac = st->rnum = st->rden = st->rfac = NULL;
	st->ballots = st->agent_voxel = NULL;
	st->initialized = 0;
}

void orc_destroy(orc_state* st)
{
	if (!st)
		return;
	free_solver(st);
	free(st->D), free(st->decay), free(st->init);
	free(st->dir_voxels), free(st->dir_values), free(st->dir_conds);
	for (int a = 0; a < 3; a++)
		for (int sd = 0; sd < 2; sd++)
			free(st->bnd_values[a][sd]), free(st->bnd_conds[a][sd]);
	free(st->bulk_supply), free(st->bulk_uptake), free(st->bulk_target);
	free(st->pos), free(st->sec), free(st->sat), free(st->upt), free(st->net), free(st->vol);
	free(st->internalized), free(st->frac_rel), free(st->active);
	free(st);
}

int orc_set_threads(orc_state* st, int threads)
{
	st->threads = threads;
	return 0;
}

static int nthreads(const orc_state* st)
{
#ifdef _OPENMP
	return st->threads > 0 ? st->threads : omp_get_max_threads();
#else
	(void)st;
	return 1;
#endif
}

/* cartesian_mesh constructor (mesh.cpp:8-28): grid = ceil((max-min)/voxel) on the
 * first `dims` axes, 1 elsewhere. */
int orc_set_mesh(orc_state* st, int dims, const int64_t bbmin[3], const int64_t bbmax[3], const uint64_t voxel[3])
{
	if (dims < 1 || dims > 3)
		return fail("dims must be 1, 2 or 3 (got %d)", dims);
	st->dims = dims;
	for (int a = 0; a < 3; a++)
	{
		st->bbmin[a] = bbmin[a];
		st->bbmax[a] = bbmax[a];
		st->voxel[a] = voxel[a];
		st->n[a] = 1;
		if (a < dims)
		{
			if (voxel[a] == 0)
				return fail("voxel shape along axis %d is zero", a);
			st->n[a] = (uint64_t)((bbmax[a] - bbmin[a] + (int64_t)voxel[a] - 1) / (int64_t)voxel[a]);
			if (st->n[a] == 0)
				return fail("empty grid along axis %d", a);
		}
	}
	st->mesh_set = 1;
	return 0;
}

int orc_get_grid(const orc_state* st, uint64_t grid[3])
{
	for (int a = 0; a < 3; a++)
		grid[a] = st->n[a];
	return 0;
}

int orc_set_substrates(orc_state* st, uint64_t S, double dt, const double* D, const double* decay, const double* init)
{
	if (S == 0)
		return fail("at least one substrate is required");
	free(st->D), free(st->decay), free(st->init);
	st->S = S;
	st->dt = dt;
	st->D = (double*)dup_array(D, S * sizeof(double));
	st->decay = (double*)dup_array(decay, S * sizeof(double));
	st->init = (double*)dup_array(init, S * sizeof(double));
	return 0;
}

/* microenvironment::dirichlet_interior_* arrays (microenvironment.h:65-69). */
int orc_set_dirichlet_interior(orc_state* st, uint64_t K, const uint64_t* voxels, const double* values,
							   const uint8_t* conditions)
{
	if (!st->mesh_set || st->S == 0)
		return fail("mesh and substrates must be set before Dirichlet nodes");
	free(st->dir_voxels), free(st->dir_values), free(st->dir_conds);
	st->K = K;
	st->dir_voxels = (uint64_t*)dup_array(voxels, K * (uint64_t)st->dims * sizeof(uint64_t));
	st->dir_values = (double*)dup_array(values, K * st->S * sizeof(double));
	st->dir_conds = (uint8_t*)dup_array(conditions, K * st->S);
	for (uint64_t k = 0; k < K; k++)
		for (int d = 0; d < st->dims; d++)
			if (st->dir_voxels[k * st->dims + d] >= st->n[d])
				return fail("Dirichlet node %llu is outside the grid", (unsigned long long)k);
	return 0;
}

/* microenvironment::dirichlet_{min,max}_boundary_{values,conditions} (microenvironment.h:72-75).
 * values == NULL removes the face (the reference leaves the pointer null). */
int orc_set_dirichlet_boundary(orc_state* st, int axis, int side, const double* values, const uint8_t* conditions)
{
	if (axis < 0 || axis > 2 || side < 0 || side > 1)
		return fail("bad boundary axis/side");
	free(st->bnd_values[axis][side]), free(st->bnd_conds[axis][side]);
	st->bnd_values[axis][side] = NULL;
	st->bnd_conds[axis][side] = NULL;
	if (values)
	{
		st->bnd_values[axis][side] = (double*)dup_array(values, st->S * sizeof(double));
		st->bnd_conds[axis][side] = (uint8_t*)dup_array(conditions, st->S);
	}
	return 0;
}

int orc_set_bulk(orc_state* st, int mode, const double* supply, const double* uptake, const double* target)
{
	free(st->bulk_supply), free(st->bulk_uptake), free(st->bulk_target);
	st->bulk_supply = st->bulk_uptake = st->bulk_target = NULL;
	st->bulk_mode = mode;
	if (mode == ORC_BULK_NONE)
		return 0;
	uint64_t cnt = st->S;
	if (mode == ORC_BULK_PER_VOXEL)
		cnt = st->S * st->n[0] * st->n[1] * st->n[2];
	else if (mode != ORC_BULK_UNIFORM)
		return fail("unknown bulk mode %d", mode);
	st->bulk_supply = (double*)dup_array(supply, cnt * sizeof(double));
	st->bulk_uptake = (double*)dup_array(uptake, cnt * sizeof(double));
	st->bulk_target = (double*)dup_array(target, cnt * sizeof(double));
	return 0;
}

/* agent_data_generic_storage SoA (agent_data_generic_storage.h:16-31). */
int orc_set_agents(orc_state* st, uint64_t A, const double* positions, const double* secretion,
				   const double* saturation, const double* uptake, const double* net_export, const double* volumes,
				   const uint8_t* is_active, const double* internalized, const double* fraction_released,
				   int compute_internalized)
{
	if (!st->mesh_set || st->S == 0)
		return fail("mesh and substrates must be set before agents");
	uint64_t S = st->S;
	free(st->pos), free(st->sec), free(st->sat), free(st->upt), free(st->net), free(st->vol);
	free(st->internalized), free(st->frac_rel), free(st->active);
	st->A = A;
	st->pos = (double*)dup_array(positions, A * (uint64_t)st->dims * sizeof(double));
	st->sec = (double*)dup_array(secretion, A * S * sizeof(double));
	st->sat = (double*)dup_array(saturation, A * S * sizeof(double));
	st->upt = (double*)dup_array(uptake, A * S * sizeof(double));
	st->net = (double*)dup_array(net_export, A * S * sizeof(double));
	st->vol = (double*)dup_array(volumes, A * sizeof(double));
	st->active = (uint8_t*)dup_array(is_active, A);
	st->internalized = (double*)calloc(A * S + 1, sizeof(double));
	if (internalized)
		memcpy(st->internalized, internalized, A * S * sizeof(double));
	st->frac_rel = (double*)calloc(A * S + 1, sizeof(double));
	if (fraction_released)
		memcpy(st->frac_rel, fraction_released, A * S * sizeof(double));
	st->compute_internalized = compute_internalized;
	/* the reference's cell_solver::resize runs on the next recompute step */
	free(st->num), free(st->den), free(st->fac), free(st->rnum), free(st->rden), free(st->rfac);
	free(st->agent_voxel);
	st->num = (double*)calloc(A * S + 1, sizeof(double));
	st->den = (double*)calloc(A * S + 1, sizeof(double));
	st->fac = (double*)calloc(A * S + 1, sizeof(double));
	st->rnum = (double*)calloc(A * S + 1, sizeof(double));
	st->rden = (double*)calloc(A * S + 1, sizeof(double));
	st->rfac = (double*)calloc(A * S + 1, sizeof(double));
	st->agent_voxel = (uint64_t*)calloc(A + 1, sizeof(uint64_t));
	st->recompute_cells = 1;
	return 0;
}

/* The reference solvers read the agent SoA by reference, so moved positions or
 * toggled is_active flags are seen on the next solve (test_cell_solver.cpp:715-763). */
int orc_update_agents(orc_state* st, const double* positions, const uint8_t* is_active)
{
	if (positions)
		memcpy(st->pos, positions, st->A * (uint64_t)st->dims * sizeof(double));
	if (is_active)
		memcpy(st->active, is_active, st->A);
	return 0;
}

/* diffusion_solver::precompute_values (openmp_solver/src/diffusion_solver.cpp:29-86).
 * Tables are [i][s] (copies = 1). */
int orc_precompute(uint64_t n, uint64_t S, uint64_t shape, uint64_t dims, double dt, const double* D,
				   const double* decay, double* b, double* e, double* c)
{
	const double h2 = (double)(shape * shape);
	for (uint64_t s = 0; s < S; s++)
		c[s] = -1 * -dt * D[s] / h2;

	for (uint64_t i = 0; i < n; i++)
		for (uint64_t s = 0; s < S; s++)
		{
			b[i * S + s] = 1 + decay[s] * dt / (double)dims + 2 * dt * D[s] / h2;
			if (i == 0 || i == n - 1)
				b[i * S + s] -= dt * D[s] / h2;
		}

	for (uint64_t s = 0; s < S; s++)
		b[s] = 1 / b[s];

	for (uint64_t i = 1; i < n; i++)
		for (uint64_t s = 0; s < S; s++)
		{
			b[i * S + s] = 1 / (b[i * S + s] - c[s] * c[s] * b[(i - 1) * S + s]);
			e[(i - 1) * S + s] = c[s] * b[(i - 1) * S + s];
		}
	return 0;
}

/* diffusion_solver::prepare + initialize (diffusion_solver.cpp:89-113),
 * cell_solver::initialize (cell_solver.cpp:394-401). */
int orc_initialize(orc_state* st)
{
	if (!st->mesh_set || st->S == 0 || !st->D)
		return fail("mesh and substrates must be set before initialize");
	if (st->initialized)
		return 0;
	const uint64_t S = st->S;
	const uint64_t V = st->n[0] * st->n[1] * st->n[2];
	st->field = (double*)malloc(V * S * sizeof(double));
	for (uint64_t v = 0; v < V; v++)
		for (uint64_t s = 0; s < S; s++)
			st->field[v * S + s] = st->init[s];
	for (int a = 0; a < st->dims; a++)
	{
		uint64_t n = st->n[a];
		st->b[a] = (double*)calloc(n * S, sizeof(double));
		st->e[a] = (double*)calloc((n > 1 ? n - 1 : 1) * S, sizeof(double));
		st->c[a] = (double*)calloc(S, sizeof(double));
		orc_precompute(n, S, st->voxel[a], (uint64_t)st->dims, st->dt, st->D, st->decay, st->b[a], st->e[a],
					   st->c[a]);
	}
	st->ballots = (uint64_t*)malloc((V + 1) * sizeof(uint64_t));
	for (uint64_t v = 0; v < V; v++)
		st->ballots[v] = 0;
	st->initialized = 1;
	return 0;
}

/* ---------------------------------------------------------------- diffusion */

/* solve_slice_x_1d / solve_slice_x_2d_and_3d (diffusion_solver.cpp:116-202):
 * one line per (y,z), all substrates of the line together. */
static void sweep_x(orc_state* st)
{
	const uint64_t S = st->S, nx = st->n[0], m = st->n[1] * st->n[2];
	const double *b = st->b[0], *e = st->e[0], *c = st->c[0];
	double* f = st->field;
#pragma omp parallel for schedule(static) num_threads(nthreads(st))
	for (uint64_t yz = 0; yz < m; yz++)
	{
		double* row = f + yz * nx * S;
		for (uint64_t i = 1; i < nx; i++)
			for (uint64_t s = 0; s < S; s++)
				row[i * S + s] = row[i * S + s] + e[(i - 1) * S + s] * row[(i - 1) * S + s];
		for (uint64_t s = 0; s < S; s++)
			row[(nx - 1) * S + s] = row[(nx - 1) * S + s] * b[(nx - 1) * S + s];
		for (int64_t i = (int64_t)nx - 2; i >= 0; i--)
			for (uint64_t s = 0; s < S; s++)
				row[i * S + s] = (row[i * S + s] + c[s] * row[(i + 1) * S + s]) * b[i * S + s];
	}
}

/* Thomas solve of `tl` independent lines that start at p[k] (k < tl) and advance by
 * `stride` per step; sub[k] is the substrate of line k.  Lines are swept together
 * inside a 48-wide tile of the merged (x,s) dimension, as the reference's y/z
 * sweeps do (diffusion_solver.cpp:390-591, 593-794). */
static void sweep_tile(double* base, uint64_t tl, uint64_t n, uint64_t stride, const uint64_t* sub, uint64_t S,
					   const double* b, const double* e, const double* c)
{
	for (uint64_t i = 1; i < n; i++)
	{
		double* cur = base + i * stride;
		double* prev = cur - stride;
		for (uint64_t k = 0; k < tl; k++)
			cur[k] = cur[k] + e[(i - 1) * S + sub[k]] * prev[k];
	}
	{
		double* last = base + (n - 1) * stride;
		for (uint64_t k = 0; k < tl; k++)
			last[k] = last[k] * b[(n - 1) * S + sub[k]];
	}
	for (int64_t i = (int64_t)n - 2; i >= 0; i--)
	{
		double* cur = base + (uint64_t)i * stride;
		double* next = cur + stride;
		for (uint64_t k = 0; k < tl; k++)
			cur[k] = (cur[k] + c[sub[k]] * next[k]) * b[(uint64_t)i * S + sub[k]];
	}
}

/* solve_slice_y_2d / solve_slice_y_3d: parallel over z, tiles over merged (x,s). */
static void sweep_y(orc_state* st)
{
	const uint64_t S = st->S, nx = st->n[0], ny = st->n[1], nz = st->n[2];
	const uint64_t xs = nx * S;
	double* f = st->field;
#pragma omp parallel for schedule(static) num_threads(nthreads(st))
	for (uint64_t z = 0; z < nz; z++)
	{
		uint64_t sub[XS_TILE];
		for (uint64_t t0 = 0; t0 < xs; t0 += XS_TILE)
		{
			uint64_t tl = xs - t0 < XS_TILE ? xs - t0 : XS_TILE;
			for (uint64_t k = 0; k < tl; k++)
				sub[k] = (t0 + k) % S;
			sweep_tile(f + z * ny * xs + t0, tl, ny, xs, sub, S, st->b[1], st->e[1], st->c[1]);
		}
	}
}

/* solve_slice_z_3d: parallel over y, tiles over merged (x,s). */
static void sweep_z(orc_state* st)
{
	const uint64_t S = st->S, nx = st->n[0], ny = st->n[1], nz = st->n[2];
	const uint64_t xs = nx * S;
	double* f = st->field;
#pragma omp parallel for schedule(static) num_threads(nthreads(st))
	for (uint64_t y = 0; y < ny; y++)
	{
		uint64_t sub[XS_TILE];
		for (uint64_t t0 = 0; t0 < xs; t0 += XS_TILE)
		{
			uint64_t tl = xs - t0 < XS_TILE ? xs - t0 : XS_TILE;
			for (uint64_t k = 0; k < tl; k++)
				sub[k] = (t0 + k) % S;
			sweep_tile(f + y * xs + t0, tl, nz, ny * xs, sub, S, st->b[2], st->e[2], st->c[2]);
		}
	}
}

/* diffusion_solver::solve dimension dispatch (diffusion_solver.cpp:797-843). */
static void diffusion(orc_state* st)
{
	sweep_x(st);
	if (st->dims >= 2)
		sweep_y(st);
	if (st->dims >= 3)
		sweep_z(st);
}

/* ---------------------------------------------------------------- Dirichlet */

/* solve_boundary on one face (dirichlet_solver.cpp:44-57). */
static void boundary_face(orc_state* st, int axis, uint64_t coord, const double* values, const uint8_t* conds)
{
	if (!values)
		return;
	const uint64_t S = st->S, nx = st->n[0], ny = st->n[1], nz = st->n[2];
	uint64_t lo[3] = { 0, 0, 0 }, hi[3] = { nx, ny, nz };
	lo[axis] = coord;
	hi[axis] = coord + 1;
	for (uint64_t z = lo[2]; z < hi[2]; z++)
		for (uint64_t y = lo[1]; y < hi[1]; y++)
			for (uint64_t x = lo[0]; x < hi[0]; x++)
			{
				double* v = st->field + S * (x + nx * (y + ny * z));
				for (uint64_t s = 0; s < S; s++)
					if (conds[s])
						v[s] = values[s];
			}
}

/* dirichlet_solver::solve (dirichlet_solver.cpp:59-93): faces x-min, x-max,
 * y-min, y-max, z-min, z-max (y/z only when the mesh has them), then interior. */
static void dirichlet(orc_state* st)
{
	for (int axis = 0; axis < st->dims; axis++)
	{
		boundary_face(st, axis, 0, st->bnd_values[axis][0], st->bnd_conds[axis][0]);
		boundary_face(st, axis, st->n[axis] - 1, st->bnd_values[axis][1], st->bnd_conds[axis][1]);
	}
	const uint64_t S = st->S, nx = st->n[0], ny = st->n[1];
	for (uint64_t k = 0; k < st->K; k++)
	{
		uint64_t idx[3] = { 0, 0, 0 };
		for (int d = 0; d < st->dims; d++)
			idx[d] = st->dir_voxels[k * st->dims + d];
		double* v = st->field + S * (idx[0] + nx * (idx[1] + ny * idx[2]));
		for (uint64_t s = 0; s < S; s++)
			if (st->dir_conds[k * S + s])
				v[s] = st->dir_values[k * S + s];
	}
}

/* ---------------------------------------------------------------- bulk */

/* bulk_solver::solve_single (bulk_solver.cpp:20-49):
 * D = (D + dt*S*T) / (1 + dt*(U+S)). */
static void bulk(orc_state* st)
{
	if (st->bulk_mode == ORC_BULK_NONE)
		return;
	const uint64_t S = st->S, V = st->n[0] * st->n[1] * st->n[2];
	const double dt = st->dt;
	const int per_voxel = st->bulk_mode == ORC_BULK_PER_VOXEL;
	double* f = st->field;
#pragma omp parallel for schedule(static) num_threads(nthreads(st))
	for (uint64_t v = 0; v < V; v++)
		for (uint64_t s = 0; s < S; s++)
		{
			uint64_t t = per_voxel ? s * V + v : s;
			const double Sr = st->bulk_supply[t];
			const double U = st->bulk_uptake[t];
			const double T = st->bulk_target[t];
			double* D = f + v * S + s;
			*D = (*D + dt * Sr * T) / (1 + dt * (U + Sr));
		}
}

/* ---------------------------------------------------------------- cells */

/* cartesian_mesh::voxel_position + linearize (mesh.cpp:37-61, 74-77). */
static int agent_voxel(const orc_state* st, uint64_t i, uint64_t* out)
{
	uint64_t idx[3] = { 0, 0, 0 };
	for (int d = 0; d < st->dims; d++)
	{
		const double p = st->pos[i * st->dims + d];
		if (!(p >= (double)st->bbmin[d]))
			return fail("agent %llu lies below the mesh along axis %d", (unsigned long long)i, d);
		idx[d] = (uint64_t)((p - (double)st->bbmin[d]) / (double)st->voxel[d]);
		if (idx[d] >= st->n[d])
			return fail("agent %llu lies outside the mesh along axis %d", (unsigned long long)i, d);
	}
	*out = idx[0] + st->n[0] * (idx[1] + st->n[1] * idx[2]);
	return 0;
}

static double voxel_volume(const orc_state* st)
{
	return (double)(st->voxel[0] * st->voxel[1] * st->voxel[2]);
}

/* compute_intermediates + clear_ballots + ballot_and_sum (cell_solver.cpp:22-129). */
static int cells_recompute(orc_state* st)
{
	const uint64_t S = st->S, A = st->A;
	const double Vv = voxel_volume(st), dt = st->dt;
	st->is_conflict = 0;
	for (uint64_t i = 0; i < A; i++)
	{
		if (!st->active[i])
			continue;
		if (agent_voxel(st, i, &st->agent_voxel[i]))
			return -1;
		for (uint64_t s = 0; s < S; s++)
		{
			const uint64_t k = i * S + s;
			st->num[k] = st->sec[k] * st->sat[k] * dt * st->vol[i] / Vv;
			st->den[k] = (st->upt[k] + st->sec[k]) * dt * st->vol[i] / Vv;
			st->fac[k] = st->net[k] * dt / Vv;
		}
	}
	for (uint64_t i = 0; i < A; i++)
	{
		if (!st->active[i])
			continue;
		st->ballots[st->agent_voxel[i]] = NO_BALLOT;
		for (uint64_t s = 0; s < S; s++)
			st->rnum[i * S + s] = st->rden[i * S + s] = st->rfac[i * S + s] = 0;
	}
	for (uint64_t i = 0; i < A; i++)
	{
		if (!st->active[i])
			continue;
		uint64_t* b = &st->ballots[st->agent_voxel[i]];
		if (*b == NO_BALLOT)
		{
			*b = i;
			for (uint64_t s = 0; s < S; s++)
			{
				st->rnum[i * S + s] += st->num[i * S + s];
				st->rden[i * S + s] += st->den[i * S + s] + 1;
				st->rfac[i * S + s] += st->fac[i * S + s];
			}
		}
		else
		{
			const uint64_t w = *b;
			st->is_conflict = 1;
			for (uint64_t s = 0; s < S; s++)
			{
				st->rnum[w * S + s] += st->num[i * S + s];
				st->rden[w * S + s] += st->den[i * S + s];
				st->rfac[w * S + s] += st->fac[i * S + s];
			}
		}
	}
	return 0;
}

/* compute_result with compute_fused / compute_densities / compute_internalized
 * (cell_solver.cpp:131-244). */
static void cells_result(orc_state* st)
{
	const uint64_t S = st->S, A = st->A;
	const double Vv = voxel_volume(st);
	double* f = st->field;
	if (st->compute_internalized && !st->is_conflict)
	{
		for (uint64_t i = 0; i < A; i++)
		{
			if (!st->active[i])
				continue;
			double* D = f + st->agent_voxel[i] * S;
			double* I = st->internalized + i * S;
			for (uint64_t s = 0; s < S; s++)
			{
				const double prev = D[s];
				D[s] = (D[s] + st->rnum[i * S + s]) / st->rden[i * S + s] + st->rfac[i * S + s];
				I[s] += Vv * (prev - D[s]);
			}
		}
		return;
	}
	for (uint64_t i = 0; i < A; i++)
	{
		if (!st->active[i] || st->ballots[st->agent_voxel[i]] != i)
			continue;
		double* D = f + st->agent_voxel[i] * S;
		for (uint64_t s = 0; s < S; s++)
			D[s] = (D[s] + st->rnum[i * S + s]) / st->rden[i * S + s] + st->rfac[i * S + s];
	}
	if (st->compute_internalized)
	{
		for (uint64_t i = 0; i < A; i++)
		{
			if (!st->active[i])
				continue;
			const double* D = f + st->agent_voxel[i] * S;
			double* I = st->internalized + i * S;
			for (uint64_t s = 0; s < S; s++)
				I[s] -= Vv * (st->num[i * S + s] - D[s] * st->den[i * S + s] + st->fac[i * S + s]);
		}
	}
}

/* simulate_secretion_and_uptake (cell_solver.cpp:246-272, 302-349). */
static int cells(orc_state* st, int recompute)
{
	if (recompute)
	{
		if (cells_recompute(st))
			return -1;
	}
	cells_result(st);
	return 0;
}

/* release_internal (cell_solver.cpp:274-289, 351-374): D += I*F/Vv, I = 0. */
int orc_release_internalized(orc_state* st, uint64_t agent)
{
	if (!st->compute_internalized)
		return 0;
	if (agent >= st->A)
		return fail("agent index out of range");
	uint64_t v;
	if (agent_voxel(st, agent, &v))
		return -1;
	const uint64_t S = st->S;
	const double Vv = voxel_volume(st);
	for (uint64_t s = 0; s < S; s++)
	{
		st->field[v * S + s] += st->internalized[agent * S + s] * st->frac_rel[agent * S + s] / Vv;
		st->internalized[agent * S + s] = 0;
	}
	return 0;
}

/* ---------------------------------------------------------------- driver */

int orc_run_phases(orc_state* st, uint32_t phases, int recompute_cells)
{
	if (orc_initialize(st))
		return -1;
	if (phases & ORC_PHASE_DIFFUSION)
		diffusion(st);
	if (phases & ORC_PHASE_DIRICHLET)
		dirichlet(st);
	if (phases & ORC_PHASE_BULK)
		bulk(st);
	if ((phases & ORC_PHASE_CELLS) && st->A > 0)
		if (cells(st, recompute_cells))
			return -1;
	return 0;
}

/* openmp_solver::solve (openmp_solver.cpp:23-40): every iteration of a call uses
 * the same recompute flag, which is cleared when the call returns. */
int orc_solve(orc_state* st, uint64_t iterations)
{
	if (orc_initialize(st))
		return -1;
	for (uint64_t it = 0; it < iterations; it++)
		if (orc_run_phases(st, ORC_PHASE_ALL, st->recompute_cells))
			return -1;
	st->recompute_cells = 0;
	return 0;
}

int orc_recompute_positional_data(orc_state* st)
{
	st->recompute_cells = 1;
	return 0;
}

int orc_get_field(const orc_state* st, double* out)
{
	if (!st->initialized)
		return fail("not initialized");
	memcpy(out, st->field, st->n[0] * st->n[1] * st->n[2] * st->S * sizeof(double));
	return 0;
}

int orc_set_field(orc_state* st, const double* in)
{
	if (orc_initialize(st))
		return -1;
	memcpy(st->field, in, st->n[0] * st->n[1] * st->n[2] * st->S * sizeof(double));
	return 0;
}

int orc_get_internalized(const orc_state* st, double* out)
{
	memcpy(out, st->internalized, st->A * st->S * sizeof(double));
	return 0;
}

/* Active agents per voxel after the last ballot (the integer histogram that the
 * ballot of cell_solver.cpp:79-129 implies). */
int orc_get_counts(const orc_state* st, uint32_t* counts)
{
	const uint64_t V = st->n[0] * st->n[1] * st->n[2];
	memset(counts, 0, V * sizeof(uint32_t));
	for (uint64_t i = 0; i < st->A; i++)
	{
		if (!st->active[i])
			continue;
		uint64_t v;
		if (agent_voxel(st, i, &v))
			return -1;
		counts[v]++;
	}
	return 0;
}

int orc_get_conflict(const orc_state* st) { return st->is_conflict; }

/* Total mass per substrate, summed in voxel order. */
int orc_mass(const orc_state* st, double* out)
{
	const uint64_t S = st->S, V = st->n[0] * st->n[1] * st->n[2];
	for (uint64_t s = 0; s < S; s++)
		out[s] = 0;
	for (uint64_t v = 0; v < V; v++)
		for (uint64_t s = 0; s < S; s++)
			out[s] += st->field[v * S + s];
	return 0;
}
