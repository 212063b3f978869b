/* Augmented Lagrangian method for LPs
 *
 *   min_x linear'x  s.t.  constraints x = rhs,  lower <= x <= upper,
 *
 * with APPROX as the inner solver.  The entry points of the reference's
 * alm.h:21-117 with the same argument meaning, ownership and return values.
 * The whole outer loop runs on the GPU (multipliers, weights and precision
 * in FP64); see acdalm_ext.h for the mixed-precision mode and statistics.
 */
#ifndef ACDALM_ALM_H
#define ACDALM_ALM_H
#include <stddef.h>
#include <stdio.h>
#include "spmv.h"
#include "approx.h"
#include "thread_pool.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct alm alm_t;
/* Copies every vector but borrows the matrix (alm.h:22-47).  linear NULL =
 * zeros; bounds NULL = -HUGE_VAL / HUGE_VAL (primal and dual).  NULL on
 * error. */
alm_t * alm_make(sparse_matrix_t * constraints,
                 size_t nrhs, const double * rhs,
                 size_t nvars, const double * linear,
                 const double * lower, const double * upper,
                 const double * lambda_lower, const double * lambda_upper);
/* Frees the instance, not the matrix; returns 0 (:48-53). */
int alm_free(alm_t *);

/* Accessors; the vectors may be modified between solves (:55-67). */
sparse_matrix_t * alm_matrix(alm_t *);
size_t alm_nrhs(alm_t *);
double * alm_rhs(alm_t *);
size_t alm_nvars(alm_t *);
double * alm_linear(alm_t *);
double * alm_lower(alm_t *);
double * alm_upper(alm_t *);
double * alm_lambda_lower(alm_t *);
double * alm_lambda_upper(alm_t *);

/* Up to niter outer iterations from x (nvars) and lambda (nconstraints),
 * both updated in place.  Stops when the largest violation < 1e-5 and the
 * inner projected gradient < 1e-5 (or the inner solve stalls).  Returns 0
 * when it stopped that way, 1 at the iteration limit, a negative
 * ACDALM_E* code on a device failure.  OUT_diagnosis (3 doubles):
 * objective, largest violation, projected-gradient norm.  The outer log
 * lines have the reference's format (:69-97). */
int alm_solve(alm_t *, size_t niter,
              double * x, size_t nvars,
              double * lambda, size_t nconstraints,
              FILE * log, double * OUT_diagnosis,
              thread_pool_t * pool);

/* Text format: a sparse matrix (spmv.h) followed by rhs, linear, lower,
 * upper, dual lower, dual upper (:98-117).  NULL on error. */
alm_t * alm_read(FILE * stream);
#ifdef __cplusplus
}
#endif
#endif
