/* Oracle: a plain-C, CPU restatement of the reference solve loop.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library, and only as the
 * checker or the timed CPU baseline -- never as the thing measured or
 * shipped.  The product (libacdalm) never links or calls it.
 *
 * Parity is pinned: with one thread, every layout (permutations, CSR, the
 * 4-row block arena, the Z-order COO) and every floating-point result
 * (step sizes, APPROX iterates, ALM iterates) is bit-identical to the
 * reference compiled from its own sources (oracle/_ref), which the tests
 * check.  With more than one thread, reductions are combined per thread in
 * a fixed order (deterministic, but not the serial bits); that mode exists
 * for the timed CPU baseline.
 */
#ifndef ACDALM_ORACLE_H
#define ACDALM_ORACLE_H
#include <stddef.h>
#include <stdint.h>

typedef struct or_matrix or_matrix_t;
typedef struct or_approx or_approx_t;
typedef struct or_alm or_alm_t;

/* Threads used by the SpMV passes and reductions (1 = serial, bit-exact). */
void or_set_threads(int nthreads);

/* spmv.c:27-92 */
or_matrix_t * or_matrix_make(size_t ncols, size_t nrows, size_t nnz,
                             const uint32_t * rows, const uint32_t * cols,
                             const double * vals, int permute);
void or_matrix_free(or_matrix_t *);
void or_matrix_dims(or_matrix_t *, size_t * nrows, size_t * ncols,
                    size_t * nnz);
void or_coo(or_matrix_t *, uint32_t * rows, uint32_t * cols, double * vals);
void or_csr(or_matrix_t *, int transpose, uint32_t * rows_indices,
            uint32_t * cols, double * vals);
size_t or_block_bytes(or_matrix_t *, int transpose, size_t * nblocks);
void or_block(or_matrix_t *, int transpose, size_t * offsets, void * arena,
              size_t bytes);
void or_perm(or_matrix_t *, int row, uint32_t * idx, uint32_t * ridx);
/* y = op(A) x over the block layout (spmv.c:159-193). */
int or_multiply(double * y, or_matrix_t *, const double * x, int transpose);
/* CSR product with the row-pair loop of spmv_csr.c:82-129 (1 RHS). */
int or_multiply_csr(double * y, or_matrix_t *, const double * x,
                    int transpose);

/* approx.c:72-216 */
or_approx_t * or_approx_make(or_matrix_t * m, size_t nrhs, const double * rhs,
                             const double * weight, size_t nvars,
                             const double * linear, const double * lower,
                             const double * upper);
void or_approx_free(or_approx_t *);
double * or_approx_vec(or_approx_t *, int which); /* 0 rhs 1 weight 2 linear
                                                     3 lower 4 upper */
int or_approx_update(or_approx_t *);
void or_approx_internals(or_approx_t *, int permuted, uint32_t * beta,
                         double * v, double * inv_v, double * rhs,
                         double * weight, double * linear, double * lower,
                         double * upper);
/* approx.c:576-708.  log_path may be NULL; trace (may be NULL) receives
 * per-iteration records of 6 doubles: value, pg, step_length, theta,
 * restarted, iteration. */
int or_approx_solve(or_approx_t *, double * x, size_t niter, double max_pg,
                    double max_value, double min_delta, const char * log_path,
                    size_t period, double * diag, double offset,
                    double * trace, size_t trace_cap);
/* approx.c:517-573 with spg_iter (mpg.inc:155-199) */
int or_mpg_solve(or_approx_t *, double * x, size_t niter, double max_pg,
                 double max_value, double min_delta, const char * log_path,
                 size_t period, double * diag, double offset);

/* alm.c:59-322 */
or_alm_t * or_alm_make(or_matrix_t * m, size_t nrhs, const double * rhs,
                       size_t nvars, const double * linear,
                       const double * lower, const double * upper,
                       const double * lambda_lower,
                       const double * lambda_upper);
void or_alm_free(or_alm_t *);
or_approx_t * or_alm_approx(or_alm_t *);
/* inner_budget caps the total APPROX iterations over the whole solve
 * ((size_t)-1 = none); *inner_used receives the count. */
int or_alm_solve(or_alm_t *, size_t niter, double * x, double * lambda,
                 const char * log_path, double * diag, size_t inner_budget,
                 size_t * inner_used);

/* Single fused epilogues, each restated from the reference and exposed so
 * the device kernels can be checked one at a time.  All vectors are in the
 * permuted coordinates of `a` (its shadow instance when permuted != 0).
 *
 * gradient_value.inc:15-81: viol = w (A x - b); returns 1/2 sum w (Ax-b)^2 */
double or_k_violation(or_approx_t * a, int permuted, const double * x,
                      double * viol);
/* gradient_value.inc:142-181: g = A' viol + c */
void or_k_gradient(or_approx_t * a, int permuted, const double * viol,
                   double * g);
/* step_project.inc:452-581: g0 = A'v0 + c, g1 = A'v1 + c,
 * zp = P(z - g1 (1-1e-6)/theta inv_v); returns max |zp| */
double or_k_gradient2_step(or_approx_t * a, int permuted, const double * v0,
                           const double * v1, const double * z, double theta,
                           double * g0, double * g1, double * zp);
/* step_project.inc:179-312 (two = 1) and :320-444 (two = 0): long step of
 * `length`, returns sum g (zp-z) + 1/2 sum (zp-z)^2 theta/length v */
double or_k_gradient_long_step(or_approx_t * a, int permuted, int two,
                               const double * v0, const double * v1,
                               const double * z, double theta, double length,
                               double * g0, double * g1, double * zp);
/* vector.inc:249-335 */
void or_k_linterp_xy(size_t n, size_t m, double * y_viol, double * x,
                     double * x_viol, const double * z, const double * z_viol,
                     double theta, double next_theta);
/* approx.c:258-278 */
double or_k_project_gradient_norm(or_approx_t * a, int permuted,
                                  const double * g, const double * x);
/* approx.c:227-256 */
double or_k_dot_diff(size_t n, const double * g, const double * z,
                     const double * zp);
#endif
