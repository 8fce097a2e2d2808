/*
 * minim_oracle.h -- CPU checker for the GPU engine (test infrastructure).
 *
 * A plain-C, FP64 restatement of the reference minim library's hot path:
 * LjNd / PhaseField / PhaseFieldUnstructured / BarAndHinge energy and
 * gradient, the generic and PhaseField constraints, and the Lbfgs / Fire /
 * GradDescent / Anneal iterations with the backtracking line search.  Only
 * tests, the smoke check and the CPU baseline leg of bench.py use it.  It is pinned against the reference's own
 * unit-test constants and against fixtures produced by the reference library
 * itself (tests/golden/).
 */
#ifndef MINIM_ORACLE_H
#define MINIM_ORACLE_H

#include <stddef.h>
#include "minim_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_inst oracle_inst;

const char* oracle_last_error(void);
int oracle_create(int kind, const void* params, const double* x0, size_t ndof,
                  const int* fixed, int nfixed, oracle_inst** out);
void oracle_destroy(oracle_inst* o);
size_t oracle_ndof(const oracle_inst* o);
/* Threads for the PhaseField evaluation and the minimisers' vector loops
 * (default 1: serial, in the reference's summation order).  More threads
 * are for timing the CPU baseline on all host cores; sums then associate
 * differently. */
void oracle_set_threads(oracle_inst* o, int nthreads);
double oracle_default_tol(const oracle_inst* o);
int oracle_set_coords(oracle_inst* o, const double* x);
int oracle_get_coords(const oracle_inst* o, double* x);
/* Energy as State::energy(x) and constrained gradient as State::gradient(x);
 * either output may be NULL.  x == NULL uses the resident coordinates. */
int oracle_energy_gradient(oracle_inst* o, const double* x, double* e, double* g);
int oracle_apply_constraints(oracle_inst* o, double* v);
int oracle_minimise(oracle_inst* o, const minim_gpu_minimiser_params* mp, minim_gpu_result* res);
/* Anneal with the C library's rand() after srand(seed), drawn in the
 * reference's order (to compare with the reference library itself). */
int oracle_anneal_libc(oracle_inst* o, const minim_gpu_minimiser_params* mp, unsigned seed,
                       minim_gpu_result* res);
/* BarAndHinge bars (2 nodes + {k,l0}) and hinges (4 nodes + {k,theta0}) in
 * the reference's element order. */
int oracle_bah_elements(const oracle_inst* o, int* nbar, const int** bars, const double** bar_par,
                        int* nhinge, const int** hinges, const double** hinge_par);
/* PhaseField kappa, kappaP (nk each), nodeVol and surfaceArea (ngrid each). */
int oracle_pf_internals(const oracle_inst* o, const double** kappa, const double** kappaP,
                        const double** node_vol, const double** surface_area, int* nk);

#ifdef __cplusplus
}
#endif
#endif
