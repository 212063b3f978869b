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
