/*
 * oracle.h -- CPU restatement of brass-pan's particle solver step.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load this library, and only as
 * the oracle the GPU results are compared with (or as the timed CPU
 * baseline), never as part of the product path.
 *
 * The state mirrors the reference's ParticleSolver device arrays
 * (brasstower/particlesolver.cuh:1075-1148): float3 arrays permuted into
 * cell-sorted order every substep, cellStart/cellEnd tables of D^3 entries
 * that are -1 for empty cells.  Arithmetic is fp32 (or fp64, see or_real) in
 * the reference's expression order; scatters run sequentially when one thread
 * is used, so a single-threaded run is deterministic.
 */
#ifndef BRASSPAN_ORACLE_H
#define BRASSPAN_ORACLE_H

#include "../include/brasspan.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Precision of the state and arithmetic: float, or double when built with
 * ORACLE_REAL_DOUBLE (liboracle64.so, the FP64 host oracle).  Field copies
 * (or_get) and state inputs (or_set_state, or_set_full_state, or_set_wind,
 * or_set_distance_params) are arrays of or_real. */
#ifdef ORACLE_REAL_DOUBLE
typedef double or_real;
#else
typedef float or_real;
#endif

typedef struct or_solver or_solver;

/* sizeof(or_real) of this build: 4 or 8. */
int or_real_size(void);

void or_set_threads(int threads);
int or_get_threads(void);

or_solver *or_create(const bp_scene_desc *scene, const bp_params *params);
void or_destroy(or_solver *s);
int or_set_params(or_solver *s, const bp_params *params);

/* ParticleSolver::update (particlesolver.cuh:772-1072), all stages of
 * params->stage_mask, `iterations` solver iterations. */
int or_update(or_solver *s, int num_substeps, float dt, int iterations, int picked_original_id,
              const float *picked_pos, const float *picked_vel);

/* Field copies (same ids as the reference build's ref_get):
 * 0 x, 1 p, 2 v (or_real [N][3]); 3 map to original, 4 map to new (int [N]);
 * 5 lambda, 6 density, 7 inverse scaled mass (or_real [N]); 8 sorted cell ids (int [N]);
 * 9 rigid rotations (or_real [B][4]); 10 rigid CMs (or_real [B][3]);
 * 11 omega, 12 normal (or_real [N][3]); 13 mass (or_real [N]); 14 phase (int [N]). */
int or_get(or_solver *s, int field, void *out);
int or_set_state(or_solver *s, const or_real *x, const or_real *v); /* sorted order */
int or_set_full_state(or_solver *s, const or_real *x, const or_real *v, const int *to_orig, const or_real *rot);
/* Overrides, in this build's precision, the textbook wind vector of the
 * parameters ([3]) and the (rest length, stiffness) pairs of the distance
 * constraints ([M][2]): finite differences of the FP64 oracle perturb them
 * without a round trip through float. */
int or_set_wind(or_solver *s, const or_real *wind);
int or_set_distance_params(or_solver *s, const or_real *params);

/* Stand-alone grid on host arrays (kernel/grid.cuh:30-99 + stable sort).
 * cell_start/cell_end: D^3 entries, -1 on entry; occupied cells are written. */
int or_grid_build(int n, const float *pos, float cell, int D, int *cell_ids, int *sorted_cell_ids,
                  int *sorted_particle_ids, int *cell_start, int *cell_end);
int or_neighbor_counts(int n, const float *sorted_pos, float cell, int D, float h,
                       const int *cell_start, const int *cell_end, int *counts);

#ifdef __cplusplus
}
#endif

#endif
