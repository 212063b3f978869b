/* APPROX: accelerated proximal coordinate descent for box-constrained
 * weighted least squares
 *
 *   min_x  sum_i weight_i/2 (A x - b)_i^2 + linear'x,  lower <= x <= upper.
 *
 * The entry points of the reference's approx/approx.h:16-128 with the same
 * argument meaning, ownership and return values.  The solve runs on the GPU
 * as one persistent kernel; see acdalm_ext.h for the extra controls.
 */
#ifndef ACDALM_APPROX_H
#define ACDALM_APPROX_H
#include <stdint.h>
#include <stddef.h>
#include <stdio.h>
#include "spmv.h"
#include "thread_pool.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct approx approx_t;

/* Copies every vector; borrows `constraints`, which must outlive the
 * instance.  weight NULL = all ones, linear NULL = zeros, bounds NULL =
 * -HUGE_VAL / HUGE_VAL.  Builds a row/column-permuted shadow copy of the
 * matrix, like the reference (approx.h:18-45, approx.c:72-92).  NULL on
 * error. */
approx_t * approx_make(sparse_matrix_t * constraints,
                       size_t nrhs, const double * rhs, const double * weight,
                       size_t nvars,
                       const double * linear,
                       const double * lower, const double * upper);
/* Frees the instance (not the borrowed matrix); NULL is ignored (:47-54). */
int approx_free(approx_t *);

/* Mutable views of the instance's vectors (:56-65). */
sparse_matrix_t * approx_matrix(approx_t *);
size_t approx_nrhs(approx_t *);
double * approx_rhs(approx_t *);
double * approx_weight(approx_t *);
size_t approx_nvars(approx_t *);
double * approx_linear(approx_t *);
double * approx_lower(approx_t *);
double * approx_upper(approx_t *);

/* Publishes changes made through the views above to the solver (step
 * sizes and the device copy).  Returns 0 (:67-72). */
int approx_update(approx_t *);

/* Minimise from x (n doubles, overwritten with the result) for up to
 * niter iterations, stopping early when the projected-gradient norm <
 * max_pg (returns 2), the objective < max_value (1), or the iterate moved
 * by less than min_delta (relative) over 100 iterations (3); 0 when niter
 * is reached.  Logs every `period` iterations to `log`; OUT_diagnosis (5
 * doubles) receives value, |g|, |pg|, delta, iterations; `offset` is added
 * to the objective; pool is ignored (:74-117).  Negative ACDALM_E* codes
 * report device failures. */
int approx_solve(double * x, size_t n, approx_t * approx, size_t niter,
                 double max_pg, double max_value, double min_delta,
                 FILE * log, size_t period,
                 double * OUT_diagnosis /* NULL or double[5] */,
                 double offset, thread_pool_t * pool);
/* Spectral projected gradient on the same instance (approx.h:118-122,
 * approx.c:517-573); returns 2. */
int mpg_solve(double * x, size_t n, approx_t * approx, size_t niter,
              double max_pg, double max_value, double min_delta,
              FILE * log, size_t period,
              double * OUT_diagnosis /* NULL or double[5] */,
              double offset, thread_pool_t * pool);
/* Same signature as the reference's randomized coordinate descent
 * (approx.h:123-127).  Runs the GPU APPROX solver: the serial random-order
 * algorithm of cd.c is not reproduced. */
int cd_solve(double * x, size_t n, approx_t * approx, size_t niter,
             double max_pg, double max_value, double min_delta,
             FILE * log, size_t period,
             double * OUT_diagnosis /* NULL or double[5] */,
             double offset, thread_pool_t * pool);
#ifdef __cplusplus
}
#endif
#endif
