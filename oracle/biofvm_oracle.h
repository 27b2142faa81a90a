/*
 * biofvm_oracle.h -- CPU restatement of the PhysiCore BioFVM reaction-diffusion
 * step (the reference's OpenMP solver), in plain C + OpenMP, FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GB300 kernels:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 * The product path (physicore_gb300) never links or calls it.
 *
 * Parity is pinned against the reference's own golden values
 * (kernels/openmp_solver/tests/test_{diffusion,bulk,dirichlet,cell}_solver.cpp),
 * extracted into tests/golden/reference_golden.json by tests/golden/extract_golden.py.
 *
 * Field layout (the reference's get_substrates_layout, diffusion_solver.h:64-83,
 * without the HWY row padding): index = s + S*(x + nx*(y + ny*z)).
 */
#ifndef PHYSICORE_BIOFVM_ORACLE_H
#define PHYSICORE_BIOFVM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_state orc_state;

/* Phases of one step, in the reference's order (openmp_solver.cpp:27-37). */
#define ORC_PHASE_DIFFUSION 1u
#define ORC_PHASE_DIRICHLET 2u
#define ORC_PHASE_BULK 4u
#define ORC_PHASE_CELLS 8u
#define ORC_PHASE_ALL 15u

/* Bulk supply/uptake table modes (bulk_functor.h:8-14 evaluated into tables). */
#define ORC_BULK_NONE 0
#define ORC_BULK_UNIFORM 1  /* arrays of length S: rate depends on s only        */
#define ORC_BULK_PER_VOXEL 2 /* arrays of length S*V, planar [s][z][y][x]        */

orc_state* orc_create(void);
void orc_destroy(orc_state* st);
const char* orc_last_error(void);

int orc_set_threads(orc_state* st, int threads);
int orc_set_mesh(orc_state* st, int dims, const int64_t bbmin[3], const int64_t bbmax[3], const uint64_t voxel[3]);
int orc_get_grid(const orc_state* st, uint64_t grid[3]);
int orc_set_substrates(orc_state* st, uint64_t S, double dt, const double* D, const double* decay, const double* init);
int orc_set_dirichlet_interior(orc_state* st, uint64_t K, const uint64_t* voxels, const double* values,
							   const uint8_t* conditions);
int orc_set_dirichlet_boundary(orc_state* st, int axis, int side, const double* values, const uint8_t* conditions);
int orc_set_bulk(orc_state* st, int mode, const double* supply, const double* uptake, const double* target);
int orc_set_agents(orc_state* st, uint64_t A, const double* positions, const double* secretion,
				   const double* saturation, const double* uptake, const double* net_export, const double* volumes,
				   const uint8_t* is_active, const double* internalized, const double* fraction_released,
				   int compute_internalized);
int orc_update_agents(orc_state* st, const double* positions, const uint8_t* is_active);
int orc_initialize(orc_state* st);
int orc_solve(orc_state* st, uint64_t iterations);
int orc_run_phases(orc_state* st, uint32_t phases, int recompute_cells);
int orc_recompute_positional_data(orc_state* st);
int orc_release_internalized(orc_state* st, uint64_t agent);

int orc_get_field(const orc_state* st, double* out);
int orc_set_field(orc_state* st, const double* in);
int orc_get_internalized(const orc_state* st, double* out);
int orc_get_counts(const orc_state* st, uint32_t* counts);
int orc_get_conflict(const orc_state* st);
int orc_mass(const orc_state* st, double* out);

/* Coefficients of one axis (diffusion_solver.cpp:29-86): b' [n*S], e [(n-1)*S], c [S]. */
int orc_precompute(uint64_t n, uint64_t S, uint64_t shape, uint64_t dims, double dt, const double* D,
				   const double* decay, double* b, double* e, double* c);

#ifdef __cplusplus
}
#endif

#endif
