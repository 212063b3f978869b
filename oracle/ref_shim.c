/* Test-infrastructure shim linked into the reference build (oracle/_ref).
 *
 * ORACLE ONLY: this file is compiled together with the reference's own C
 * sources by oracle/Makefile.  Only the tests, the smoke check and the CPU
 * baseline leg of bench.py may load the result.
 *
 * It does three things:
 *
 *  1. Defines cd_solve as a forwarder to the reference's approx_solve (same
 *     signature, approx/approx.h:113-127).  alm_solve hard-codes cd_solve as
 *     its inner solver (alm.c:255); with this forwarder the reference runs
 *     ALM over its own APPROX, which is the loop being rebuilt.  cd.c is not
 *     compiled.  An optional global budget of inner iterations (the "20,000
 *     inner iterations" stopping rule of the small CPU workload) is enforced
 *     by shrinking niter and counting OUT_diagnosis[4].
 *
 *  2. Exposes read-only views of the reference's internal layouts (CSR,
 *     4-row block arena, permutations, step-size vectors) so the tests can
 *     compare them byte for byte with the new implementation.
 *
 *  3. Wraps alm_solve / approx_solve with a log file path and a thread count
 *     so they can be driven from Python through ctypes.
 */
#include <assert.h>
#include <math.h>
#include <setjmp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "alm.h"
#include "approx/approx.h"
#include "spmv/spmv_internal.h"
#include "thread_pool/thread_pool.h"

/* ---- 1. cd_solve -> approx_solve, with an optional inner budget ---- */

static size_t inner_budget = (size_t)-1;
static size_t inner_used = 0;

/* Optional relative-KKT stop (the metric's stop rule), armed by
 * ref_alm_solve_kkt: at the entry of every inner solve after the first --
 * i.e. at the start of outer iteration k > 0, where x is the previous inner
 * solve's output and lambda has just been updated (alm.c:247-287) -- the
 * residuals of (x, lambda) are computed with the reference's own SpMV:
 *
 *   primal = |A x - b|_2 / (1 + |b|_2)
 *   dual   = |x - P[l,u](x - r)|_2 / (1 + |c|_2),  r = c - A' lambda
 *            (the inner problem's linear term, approx_linear)
 *   gap    = |c'x - (b'lambda + sum_j min(l_j r_j, u_j r_j))|
 *            / (1 + |c'x| + |dual objective|)
 *
 * (b'lambda is the offset alm.c passes in).  When their maximum is at most
 * the tolerance the solve is left by longjmp back into ref_alm_solve_kkt:
 * x and lambda are the caller's arrays, so they hold exactly the point that
 * was checked. */
static struct {
        int armed;
        double tol;
        const double * lambda;
        const double * c0;
        sparse_matrix_t * a;
        size_t calls;
        jmp_buf back;
        double last[4];  /* primal, dual, gap, objective of the last check */
} kkt;

static void kkt_terms(const double * x, approx_t * approx, double offset,
                      double out[4])
{
        size_t m = approx_nrhs(approx), n = approx_nvars(approx);
        const double * b = approx_rhs(approx);
        const double * r = approx_linear(approx);
        const double * l = approx_lower(approx);
        const double * u = approx_upper(approx);
        double * ax = calloc(m ? m : 1, sizeof(double));
        assert(0 == sparse_matrix_multiply(ax, m, kkt.a, x, n, 0, NULL));
        double rr = 0, bb = 0;
        for (size_t i = 0; i < m; i++) {
                double d = ax[i] - b[i];
                rr += d * d;
                bb += b[i] * b[i];
        }
        free(ax);
        double dd = 0, cc = 0, cx = 0, box = 0;
        for (size_t j = 0; j < n; j++) {
                double p = fmax(l[j], fmin(x[j] - r[j], u[j]));
                double d = x[j] - p;
                dd += d * d;
                cc += kkt.c0[j] * kkt.c0[j];
                cx += kkt.c0[j] * x[j];
                double lo = isfinite(l[j]) ? l[j] * r[j] : HUGE_VAL;
                double hi = isfinite(u[j]) ? u[j] * r[j] : HUGE_VAL;
                double t = fmin(lo, hi);
                box += isfinite(t) ? t : 0.0;
        }
        double dobj = offset + box;
        out[0] = sqrt(rr) / (1 + sqrt(bb));
        out[1] = sqrt(dd) / (1 + sqrt(cc));
        out[2] = fabs(cx - dobj) / (1 + fabs(cx) + fabs(dobj));
        out[3] = cx;
}

void ref_set_inner_budget(size_t budget)
{
        inner_budget = budget;
        inner_used = 0;
}

size_t ref_inner_used(void)
{
        return inner_used;
}

int cd_solve(double * x, size_t n, approx_t * approx, size_t niter,
             double max_pg, double max_value, double min_delta,
             FILE * log, size_t period, double * OUT_diagnosis,
             double offset, thread_pool_t * pool)
{
        double local[5];
        double * diag = (OUT_diagnosis != NULL) ? OUT_diagnosis : local;
        if (kkt.armed && kkt.calls++ > 0) {
                kkt_terms(x, approx, offset, kkt.last);
                double rk = fmax(kkt.last[0], fmax(kkt.last[1], kkt.last[2]));
                if (rk <= kkt.tol)
                        longjmp(kkt.back, 1);
        }
        if (inner_budget != (size_t)-1) {
                size_t left = (inner_used < inner_budget)
                        ? inner_budget - inner_used : 0;
                if (niter > left)
                        niter = left;
        }
        int reason = approx_solve(x, n, approx, niter, max_pg, max_value,
                                  min_delta, log, period, diag, offset, pool);
        /* approx.c:701 reports i+1; the loop ran niter times when it
         * exhausted the budget (reason 0), else i+1 times. */
        size_t ran = (reason == 0) ? niter : (size_t)diag[4];
        inner_used += ran;
        return reason;
}

/* ---- 2. read-only views of the internal layouts ---- */

void ref_matrix_dims(sparse_matrix_t * m, size_t * nrows, size_t * ncols,
                     size_t * nnz)
{
        *nrows = m->nrows;
        *ncols = m->ncolumns;
        *nnz = m->nnz;
}

void ref_coo(sparse_matrix_t * m, uint32_t * rows, uint32_t * cols,
             double * vals)
{
        memcpy(rows, m->rows, m->nnz * sizeof(uint32_t));
        memcpy(cols, m->columns, m->nnz * sizeof(uint32_t));
        memcpy(vals, m->values, m->nnz * sizeof(double));
}

void ref_csr(sparse_matrix_t * m, int transpose, uint32_t * rows_indices,
             uint32_t * cols, double * vals)
{
        const struct csr * csr = transpose ? &m->transpose : &m->matrix;
        memcpy(rows_indices, csr->rows_indices,
               (csr->nrows + 1) * sizeof(uint32_t));
        memcpy(cols, csr->columns, m->nnz * sizeof(uint32_t));
        memcpy(vals, csr->values, m->nnz * sizeof(double));
}

/* Size in bytes of the block arena that the blocks actually occupy: the
 * last block's offset plus its 64-byte-rounded size (spmv_block.c:100-114,
 * :164-168). */
size_t ref_block_bytes(sparse_matrix_t * m, int transpose, size_t * nblocks)
{
        const struct block_matrix * b = transpose ? &m->block_transpose
                                                  : &m->block;
        *nblocks = b->nblocks;
        if (b->nblocks == 0)
                return 0;
        const struct matrix_subblock * last = (const struct matrix_subblock *)
                ((const char *)b->blocks + b->block_offsets[b->nblocks - 1]);
        size_t bytes = sizeof(struct matrix_subblock)
                + (sizeof(double) + sizeof(uint32_t)) * 4 * last->nnz;
        bytes = (bytes + 63) & ~(size_t)63;
        return b->block_offsets[b->nblocks - 1] + bytes;
}

void ref_block(sparse_matrix_t * m, int transpose, size_t * offsets,
               void * arena, size_t bytes)
{
        const struct block_matrix * b = transpose ? &m->block_transpose
                                                  : &m->block;
        memcpy(offsets, b->block_offsets, b->nblocks * sizeof(size_t));
        if (bytes)
                memcpy(arena, b->blocks, bytes);
}

void ref_perm(sparse_matrix_t * m, int row, uint32_t * idx, uint32_t * ridx)
{
        const sparse_permutation_t * p = row ? &m->row_permutation
                                             : &m->col_permutation;
        memcpy(idx, p->idx, p->n * sizeof(uint32_t));
        memcpy(ridx, p->ridx, p->n * sizeof(uint32_t));
}

/* Field-for-field view of the reference's private struct approx
 * (approx/approx.c:10-24); the layout has to be the same to read it. */
struct ref_approx_view {
        size_t nrhs, nvars;
        sparse_matrix_t * matrix;
        double * rhs;
        double * weight;
        double * linear;
        double * lower, * upper;
        uint32_t * beta;
        double * v;
        double * inv_v;
        struct ref_approx_view * permuted;
};

sparse_matrix_t * ref_approx_permuted_matrix(approx_t * a)
{
        struct ref_approx_view * v = (struct ref_approx_view *)a;
        return v->permuted ? v->permuted->matrix : NULL;
}

/* beta[nrhs], v[nvars], inv_v[nvars], plus the permuted copies of
 * rhs/weight (rows) and linear/lower/upper (columns) of the shadow
 * instance when permuted != 0. */
void ref_approx_internals(approx_t * a, int permuted, uint32_t * beta,
                          double * v, double * inv_v, double * rhs,
                          double * weight, double * linear, double * lower,
                          double * upper)
{
        struct ref_approx_view * s = (struct ref_approx_view *)a;
        if (permuted)
                s = s->permuted;
        memcpy(beta, s->beta, s->nrhs * sizeof(uint32_t));
        memcpy(v, s->v, s->nvars * sizeof(double));
        memcpy(inv_v, s->inv_v, s->nvars * sizeof(double));
        memcpy(rhs, s->rhs, s->nrhs * sizeof(double));
        memcpy(weight, s->weight, s->nrhs * sizeof(double));
        memcpy(linear, s->linear, s->nvars * sizeof(double));
        memcpy(lower, s->lower, s->nvars * sizeof(double));
        memcpy(upper, s->upper, s->nvars * sizeof(double));
}

/* ---- 3. solve wrappers with a log path and a thread count ---- */

static thread_pool_t * make_pool(int nthreads)
{
        return (nthreads > 0) ? thread_pool_init((unsigned)nthreads) : NULL;
}

int ref_alm_solve(alm_t * alm, size_t niter, double * x, double * lambda,
                  const char * log_path, double * diag, int nthreads)
{
        FILE * log = (log_path != NULL) ? fopen(log_path, "w") : NULL;
        thread_pool_t * pool = make_pool(nthreads);
        int r = alm_solve(alm, niter, x, alm_nvars(alm), lambda,
                          alm_nrhs(alm), log, diag, pool);
        thread_pool_free(pool);
        if (log != NULL)
                fclose(log);
        return r;
}

/* alm_solve stopped at relative KKT <= tol, checked at the start of every
 * outer iteration after the first (see cd_solve above).  Returns 0 when the
 * tolerance was reached, else alm_solve's own return value; kkt_out (4
 * doubles) receives primal, dual, gap and c'x of the last check, outer_out
 * the outer iterations started.  On the stop the state alm_solve allocated
 * for itself (one vector of nrhs doubles) is not freed: this is a fixture
 * generator that runs once. */
int ref_alm_solve_kkt(alm_t * alm, size_t niter, double * x, double * lambda,
                      double tol, double * kkt_out, size_t * outer_out,
                      int nthreads)
{
        thread_pool_t * pool = make_pool(nthreads);
        kkt.armed = 1;
        kkt.tol = tol;
        kkt.lambda = lambda;
        kkt.c0 = alm_linear(alm);
        kkt.a = alm_matrix(alm);
        kkt.calls = 0;
        memset(kkt.last, 0, sizeof(kkt.last));
        volatile int r;
        volatile size_t outer;
        if (setjmp(kkt.back) == 0) {
                r = alm_solve(alm, niter, x, alm_nvars(alm), lambda,
                              alm_nrhs(alm), NULL, NULL, pool);
                outer = kkt.calls;
        } else {
                r = 0;
                outer = kkt.calls - 1;  /* the check ran before this one */
        }
        kkt.armed = 0;
        *outer_out = outer;
        memcpy(kkt_out, kkt.last, sizeof(kkt.last));
        thread_pool_free(pool);
        return r;
}

int ref_approx_solve(approx_t * a, double * x, size_t niter, double max_pg,
                     double max_value, double min_delta,
                     const char * log_path, size_t period, double * diag,
                     double offset, int nthreads)
{
        FILE * log = (log_path != NULL) ? fopen(log_path, "w") : NULL;
        thread_pool_t * pool = make_pool(nthreads);
        int r = approx_solve(x, approx_nvars(a), a, niter, max_pg, max_value,
                             min_delta, log, period, diag, offset, pool);
        thread_pool_free(pool);
        if (log != NULL)
                fclose(log);
        return r;
}

int ref_mpg_solve(approx_t * a, double * x, size_t niter, double max_pg,
                  double max_value, double min_delta, const char * log_path,
                  size_t period, double * diag, double offset, int nthreads)
{
        FILE * log = (log_path != NULL) ? fopen(log_path, "w") : NULL;
        thread_pool_t * pool = make_pool(nthreads);
        int r = mpg_solve(x, approx_nvars(a), a, niter, max_pg, max_value,
                          min_delta, log, period, diag, offset, pool);
        thread_pool_free(pool);
        if (log != NULL)
                fclose(log);
        return r;
}
