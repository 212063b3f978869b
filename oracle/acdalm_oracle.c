/* Oracle: plain-C CPU restatement of the reference's ALM + APPROX solve loop.
 *
 * TEST INFRASTRUCTURE ONLY -- see acdalm_oracle.h.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * Every function cites the reference file:line it restates.  The arithmetic
 * follows the reference operation for operation (two-lane "pair"
 * accumulators where the reference uses its v2d vectors, the same
 * association of products, no fused multiply-add), so that with one thread
 * the results are bit-identical to the reference built from its sources.
 */
#define _GNU_SOURCE
#include "acdalm_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;

void or_set_threads(int nthreads)
{
        g_threads = (nthreads < 1) ? 1 : (nthreads > 256 ? 256 : nthreads);
}

/* huge_alloc/huge_alloc.default.inc:6-27: zeroed, 64-byte aligned, with 16
 * zero bytes past the end so two-lane loops over an odd length read a 0. */
static void * zalloc(size_t n, size_t size)
{
        size_t bytes = n * size + 16;
        bytes = (bytes + 63) & ~(size_t)63;
        void * p = aligned_alloc(64, bytes);
        if (p == NULL) {
                fprintf(stderr, "oracle: out of memory\n");
                abort();
        }
        memset(p, 0, bytes);
        return p;
}

static double * dup_or(const double * src, size_t n, double missing)
{
        double * out = zalloc(n, sizeof(double));
        for (size_t i = 0; i < n; i++)
                out[i] = (src != NULL) ? src[i] : missing;
        return out;
}

/* SSE2 MAXPD / MINPD lane rule (the second operand wins ties and NaN),
 * as used by step_project.inc and approx.c:272-273. */
static inline double maxpd(double a, double b) { return (a > b) ? a : b; }
static inline double minpd(double a, double b) { return (a < b) ? a : b; }

/* ------------------------------------------------------------------ */
/* Layouts: permutation, CSR, 4-row blocks, Z-order COO                */
/* ------------------------------------------------------------------ */

typedef struct {
        size_t nrows;
        uint32_t * rows_indices; /* nrows+1 */
        uint32_t * columns;
        double * values;
} csr_t;

typedef struct {
        size_t nrows, nblocks;
        size_t * offsets;
        unsigned char * arena;
        size_t bytes;
} blockm_t;

typedef struct {
        size_t n;
        uint32_t * idx, * ridx;
} perm_t;

struct or_matrix {
        size_t ncols, nrows, nnz;
        uint32_t * rows, * cols;
        double * vals;
        csr_t csr, csr_t_;
        blockm_t block, block_t;
        perm_t rperm, cperm;
};

#define BLK 4           /* SPMV_BLOCK_SIZE, spmv_block.h:3-5 */
#define BLK_RING 16     /* SPMV_BLOCK_BUFFER_SIZE, spmv_block.c:143-145 */
#define BLK_HDR 32      /* sizeof(struct matrix_subblock), spmv_block.h:9-17 */
#define SORT_SCOPE 256  /* PERMUTATION_SORTING_SCOPE, permutation.c:59-61 */

static void perm_identity(perm_t * p, size_t n)
{
        p->n = n;
        p->idx = calloc(n ? n : 1, sizeof(uint32_t));
        p->ridx = calloc(n ? n : 1, sizeof(uint32_t));
        for (size_t i = 0; i < n; i++)
                p->idx[i] = p->ridx[i] = (uint32_t)i;
}

typedef struct {
        uint32_t count, index;
} count_pair_t;

static int cmp_count_pair(const void * a, const void * b)
{
        const count_pair_t * x = a, * y = b;
        if (x->count != y->count)
                return (x->count < y->count) ? -1 : 1;
        return (x->index < y->index) ? -1 : (x->index > y->index);
}

/* permutation.c:63-125 (default build: no PERMUTATION_FIRST_NZ, no
 * shuffle): count nonzeros per row (or column), sort each window of 256
 * by (count, original index); idx = new -> old, ridx = old -> new. */
static void perm_init(perm_t * p, const uint32_t * keys, size_t nnz, size_t n)
{
        count_pair_t * pairs = calloc(n ? n : 1, sizeof(count_pair_t));
        for (size_t i = 0; i < n; i++)
                pairs[i].index = (uint32_t)i;
        for (size_t i = 0; i < nnz; i++)
                pairs[keys[i]].count++;
        for (size_t i = 0; i < n; i += SORT_SCOPE) {
                size_t m = (n - i < SORT_SCOPE) ? n - i : SORT_SCOPE;
                qsort(pairs + i, m, sizeof(count_pair_t), cmp_count_pair);
        }
        p->n = n;
        p->idx = calloc(n ? n : 1, sizeof(uint32_t));
        p->ridx = calloc(n ? n : 1, sizeof(uint32_t));
        for (size_t i = 0; i < n; i++) {
                p->idx[i] = pairs[i].index;
                p->ridx[pairs[i].index] = (uint32_t)i;
        }
        free(pairs);
}

typedef struct {
        uint64_t key;
        uint32_t pos;
} keyed_t;

static int cmp_keyed(const void * a, const void * b)
{
        const keyed_t * x = a, * y = b;
        return (x->key < y->key) ? -1 : (x->key > y->key);
}

/* spmv_csr.c:27-80: order entries by (row << 32 | column) (keys are
 * unique), rows_indices[r+1] = 1 + last position of row r, then a running
 * maximum fills empty rows. */
static void csr_build(const struct or_matrix * m, csr_t * c, int transpose)
{
        size_t nnz = m->nnz;
        size_t n = transpose ? m->ncols : m->nrows;
        keyed_t * e = calloc(nnz ? nnz : 1, sizeof(keyed_t));
        for (size_t i = 0; i < nnz; i++) {
                uint64_t r = transpose ? m->cols[i] : m->rows[i];
                uint64_t col = transpose ? m->rows[i] : m->cols[i];
                e[i].key = (r << 32) | col;
                e[i].pos = (uint32_t)i;
        }
        qsort(e, nnz, sizeof(keyed_t), cmp_keyed);
        c->nrows = n;
        c->rows_indices = calloc(n + 1, sizeof(uint32_t));
        c->columns = zalloc(nnz, sizeof(uint32_t));
        c->values = zalloc(nnz, sizeof(double));
        for (size_t i = 0; i < nnz; i++) {
                uint32_t r = (uint32_t)(e[i].key >> 32);
                c->rows_indices[r + 1] = (uint32_t)(i + 1);
                c->columns[i] = (uint32_t)(e[i].key & 0xffffffffu);
                c->values[i] = m->vals[e[i].pos];
        }
        uint32_t run = 0;
        for (size_t i = 0; i <= n; i++) {
                if (c->rows_indices[i] > run)
                        run = c->rows_indices[i];
                c->rows_indices[i] = run;
        }
        free(e);
}

static size_t block_size_bytes(size_t nnz)
{
        size_t b = BLK_HDR + (sizeof(double) + sizeof(uint32_t)) * BLK * nnz;
        return (b + 63) & ~(size_t)63;
}

/* spmv_block.c:58-149: one block per 4 consecutive rows; slot j of row r
 * at position j*4 + r; width = the longest row; padding slots (value 0 --
 * and any stored 0.0 entry) take their column from a 16-entry ring of the
 * columns seen while scanning the block backwards.  Blocks are packed in a
 * zeroed arena at 64-byte rounded offsets. */
static void block_build(const csr_t * c, blockm_t * b)
{
        size_t nrows = c->nrows;
        size_t nblocks = (nrows + BLK - 1) / BLK;
        b->nrows = nrows;
        b->nblocks = nblocks;
        b->offsets = calloc(nblocks ? nblocks : 1, sizeof(size_t));
        size_t total = 0;
        for (size_t blk = 0; blk < nblocks; blk++) {
                size_t start = blk * BLK, width = 0;
                for (size_t r = start; r < start + BLK && r < nrows; r++) {
                        size_t len = c->rows_indices[r + 1]
                                - c->rows_indices[r];
                        if (len > width)
                                width = len;
                }
                b->offsets[blk] = total;
                total += block_size_bytes(width);
        }
        b->bytes = total;
        b->arena = zalloc(total, 1);
        for (size_t blk = 0; blk < nblocks; blk++) {
                unsigned char * base = b->arena + b->offsets[blk];
                size_t start = blk * BLK;
                size_t nr = (nrows - start < BLK) ? nrows - start : BLK;
                size_t width = 0;
                for (size_t r = 0; r < nr; r++) {
                        size_t len = c->rows_indices[start + r + 1]
                                - c->rows_indices[start + r];
                        if (len > width)
                                width = len;
                }
                size_t slots = BLK * width;
                double * vals = (double *)(base + BLK_HDR);
                uint32_t * cols = (uint32_t *)(vals + slots);
                for (size_t r = 0; r < nr; r++) {
                        size_t k = r;
                        for (uint32_t j = c->rows_indices[start + r];
                             j < c->rows_indices[start + r + 1];
                             j++, k += BLK) {
                                cols[k] = c->columns[j];
                                vals[k] = c->values[j];
                        }
                }
                uint32_t ring[BLK_RING] = {0};
                size_t rd = 0, wr = 0;
                for (size_t k = slots; k-- > 0;) {
                        if (vals[k] == 0) {
                                cols[k] = ring[rd];
                                rd = (rd + 1) % BLK_RING;
                        } else {
                                ring[wr] = cols[k];
                                wr = (wr + 1) % BLK_RING;
                        }
                }
                uint32_t * hdr = (uint32_t *)base;
                hdr[0] = (uint32_t)width;
                hdr[1] = (uint32_t)start;
                hdr[2] = (uint32_t)nr;
        }
}

/* spmv.swizzle.inc:1-12: column bit i -> key bit 2i, row bit i -> 2i+1. */
static uint64_t morton(uint32_t col, uint32_t row)
{
        uint64_t k = 0;
        for (unsigned i = 0; i < 32; i++) {
                k |= (uint64_t)((col >> i) & 1u) << (2 * i);
                k |= (uint64_t)((row >> i) & 1u) << (2 * i + 1);
        }
        return k;
}

/* spmv.swizzle.inc:14-52: reorder the COO triplets by Morton key. */
static void coo_swizzle(struct or_matrix * m)
{
        size_t nnz = m->nnz;
        keyed_t * e = calloc(nnz ? nnz : 1, sizeof(keyed_t));
        for (size_t i = 0; i < nnz; i++) {
                e[i].key = morton(m->cols[i], m->rows[i]);
                e[i].pos = (uint32_t)i;
        }
        qsort(e, nnz, sizeof(keyed_t), cmp_keyed);
        uint32_t * r = zalloc(nnz, sizeof(uint32_t));
        uint32_t * c = zalloc(nnz, sizeof(uint32_t));
        double * v = zalloc(nnz, sizeof(double));
        for (size_t i = 0; i < nnz; i++) {
                r[i] = m->rows[e[i].pos];
                c[i] = m->cols[e[i].pos];
                v[i] = m->vals[e[i].pos];
        }
        free(m->rows);
        free(m->cols);
        free(m->vals);
        m->rows = r;
        m->cols = c;
        m->vals = v;
        free(e);
}

/* spmv.c:27-92 */
or_matrix_t * or_matrix_make(size_t ncols, size_t nrows, size_t nnz,
                             const uint32_t * rows, const uint32_t * cols,
                             const double * vals, int permute)
{
        struct or_matrix * m = calloc(1, sizeof(*m));
        m->ncols = ncols;
        m->nrows = nrows;
        m->nnz = nnz;
        m->rows = zalloc(nnz, sizeof(uint32_t));
        m->cols = zalloc(nnz, sizeof(uint32_t));
        m->vals = zalloc(nnz, sizeof(double));
        memcpy(m->rows, rows, nnz * sizeof(uint32_t));
        memcpy(m->cols, cols, nnz * sizeof(uint32_t));
        memcpy(m->vals, vals, nnz * sizeof(double));
        if (permute) {
                perm_init(&m->rperm, m->rows, nnz, nrows);
                perm_init(&m->cperm, m->cols, nnz, ncols);
                for (size_t i = 0; i < nnz; i++) {
                        m->rows[i] = m->rperm.ridx[m->rows[i]];
                        m->cols[i] = m->cperm.ridx[m->cols[i]];
                }
        } else {
                perm_identity(&m->rperm, nrows);
                perm_identity(&m->cperm, ncols);
        }
        csr_build(m, &m->csr, 0);
        csr_build(m, &m->csr_t_, 1);
        block_build(&m->csr, &m->block);
        block_build(&m->csr_t_, &m->block_t);
        coo_swizzle(m);
        return m;
}

static void csr_free(csr_t * c)
{
        free(c->rows_indices);
        free(c->columns);
        free(c->values);
}

static void block_free(blockm_t * b)
{
        free(b->offsets);
        free(b->arena);
}

void or_matrix_free(or_matrix_t * m)
{
        if (m == NULL)
                return;
        free(m->rows);
        free(m->cols);
        free(m->vals);
        csr_free(&m->csr);
        csr_free(&m->csr_t_);
        block_free(&m->block);
        block_free(&m->block_t);
        free(m->rperm.idx);
        free(m->rperm.ridx);
        free(m->cperm.idx);
        free(m->cperm.ridx);
        free(m);
}

void or_matrix_dims(or_matrix_t * m, size_t * nrows, size_t * ncols,
                    size_t * nnz)
{
        *nrows = m->nrows;
        *ncols = m->ncols;
        *nnz = m->nnz;
}

void or_coo(or_matrix_t * m, uint32_t * rows, uint32_t * cols, double * vals)
{
        memcpy(rows, m->rows, m->nnz * sizeof(uint32_t));
        memcpy(cols, m->cols, m->nnz * sizeof(uint32_t));
        memcpy(vals, m->vals, m->nnz * sizeof(double));
}

void or_csr(or_matrix_t * m, int transpose, uint32_t * rows_indices,
            uint32_t * cols, double * vals)
{
        const csr_t * c = transpose ? &m->csr_t_ : &m->csr;
        memcpy(rows_indices, c->rows_indices,
               (c->nrows + 1) * sizeof(uint32_t));
        memcpy(cols, c->columns, m->nnz * sizeof(uint32_t));
        memcpy(vals, c->values, m->nnz * sizeof(double));
}

size_t or_block_bytes(or_matrix_t * m, int transpose, size_t * nblocks)
{
        const blockm_t * b = transpose ? &m->block_t : &m->block;
        *nblocks = b->nblocks;
        return b->bytes;
}

void or_block(or_matrix_t * m, int transpose, size_t * offsets, void * arena,
              size_t bytes)
{
        const blockm_t * b = transpose ? &m->block_t : &m->block;
        memcpy(offsets, b->offsets, b->nblocks * sizeof(size_t));
        if (bytes)
                memcpy(arena, b->arena, bytes);
}

void or_perm(or_matrix_t * m, int row, uint32_t * idx, uint32_t * ridx)
{
        const perm_t * p = row ? &m->rperm : &m->cperm;
        memcpy(idx, p->idx, p->n * sizeof(uint32_t));
        memcpy(ridx, p->ridx, p->n * sizeof(uint32_t));
}

/* ------------------------------------------------------------------ */
/* Block products (spmv_block.c:160-320)                              */
/* ------------------------------------------------------------------ */

static inline const unsigned char * block_at(const blockm_t * b, size_t i)
{
        return b->arena + b->offsets[i];
}

/* mult_subblock, spmv_block.c:160-194: per row, acc += value * x[col]
 * over every slot (padding included), then store the live rows. */
static void block_mult_range(const blockm_t * b, size_t from, size_t to,
                             double * out, const double * x)
{
        for (size_t i = from; i < to; i++) {
                const unsigned char * base = block_at(b, i);
                const uint32_t * hdr = (const uint32_t *)base;
                size_t width = hdr[0];
                const double * vals = (const double *)(base + BLK_HDR);
                const uint32_t * cols = (const uint32_t *)(vals + BLK * width);
                double acc[BLK] = {0, 0, 0, 0};
                for (size_t s = 0; s < width; s++)
                        for (int r = 0; r < BLK; r++)
                                acc[r] = acc[r] + vals[s * BLK + r]
                                        * x[cols[s * BLK + r]];
                for (uint32_t r = 0; r < hdr[2]; r++)
                        out[hdr[1] + r] = acc[r];
        }
}

/* mult2_subblock, spmv_block.c:196-254 */
static void block_mult2_range(const blockm_t * b, size_t from, size_t to,
                              double * out0, double * out1,
                              const double * x0, const double * x1)
{
        for (size_t i = from; i < to; i++) {
                const unsigned char * base = block_at(b, i);
                const uint32_t * hdr = (const uint32_t *)base;
                size_t width = hdr[0];
                const double * vals = (const double *)(base + BLK_HDR);
                const uint32_t * cols = (const uint32_t *)(vals + BLK * width);
                double a0[BLK] = {0, 0, 0, 0}, a1[BLK] = {0, 0, 0, 0};
                for (size_t s = 0; s < width; s++)
                        for (int r = 0; r < BLK; r++) {
                                double v = vals[s * BLK + r];
                                uint32_t c = cols[s * BLK + r];
                                a0[r] = a0[r] + v * x0[c];
                                a1[r] = a1[r] + v * x1[c];
                        }
                for (uint32_t r = 0; r < hdr[2]; r++) {
                        out0[hdr[1] + r] = a0[r];
                        out1[hdr[1] + r] = a1[r];
                }
        }
}

/* Row range [begin, end) covered by blocks [from, to). */
static void block_rows(const blockm_t * b, size_t from, size_t to,
                       size_t * begin, size_t * end)
{
        *begin = from * BLK;
        *end = (to * BLK < b->nrows) ? to * BLK : b->nrows;
}

/* Static split of [0, n) into `parts` contiguous chunks (thread t gets
 * chunk t); a multiple of `align` per chunk boundary. */
static void split(size_t n, int parts, int t, size_t align, size_t * lo,
                  size_t * hi)
{
        size_t units = (n + align - 1) / align;
        size_t per = units / (size_t)parts, rem = units % (size_t)parts;
        size_t a = (size_t)t * per + ((size_t)t < rem ? (size_t)t : rem);
        size_t b = a + per + ((size_t)t < rem ? 1 : 0);
        *lo = a * align;
        *hi = b * align;
        if (*lo > n) *lo = n;
        if (*hi > n) *hi = n;
}

int or_multiply(double * y, or_matrix_t * m, const double * x, int transpose)
{
        const blockm_t * b = transpose ? &m->block_t : &m->block;
#pragma omp parallel for schedule(static) num_threads(g_threads) if (g_threads > 1)
        for (int t = 0; t < g_threads; t++) {
                size_t lo, hi;
                split(b->nblocks, g_threads, t, 1, &lo, &hi);
                block_mult_range(b, lo, hi, y, x);
        }
        return 0;
}

/* mult_csr, spmv_csr.c:82-129: rows in pairs, each row accumulated in its
 * own sequential sum. */
int or_multiply_csr(double * y, or_matrix_t * m, const double * x,
                    int transpose)
{
        const csr_t * c = transpose ? &m->csr_t_ : &m->csr;
        for (size_t r = 0; r < c->nrows; r++) {
                double acc = 0;
                for (uint32_t j = c->rows_indices[r];
                     j < c->rows_indices[r + 1]; j++)
                        acc += c->values[j] * x[c->columns[j]];
                y[r] = acc;
        }
        return 0;
}

/* ------------------------------------------------------------------ */
/* APPROX instance (approx.c:10-216)                                  */
/* ------------------------------------------------------------------ */

struct or_approx {
        size_t nrhs, nvars;
        or_matrix_t * matrix;
        double * rhs, * weight, * linear, * lower, * upper;
        uint32_t * beta;
        double * v, * inv_v;
        struct or_approx * permuted;
        int owns_matrix;
};

static or_approx_t * approx_make_1(or_matrix_t * m, size_t nrhs,
                                   const double * rhs, const double * weight,
                                   size_t nvars, const double * linear,
                                   const double * lower, const double * upper)
{
        or_approx_t * a = calloc(1, sizeof(*a));
        a->nrhs = nrhs;
        a->nvars = nvars;
        a->matrix = m;
        a->rhs = dup_or(rhs, nrhs, 0);
        a->weight = dup_or(weight, nrhs, 1);
        a->linear = dup_or(linear, nvars, 0);
        a->lower = dup_or(lower, nvars, -HUGE_VAL);
        a->upper = dup_or(upper, nvars, HUGE_VAL);
        a->beta = zalloc(nrhs, sizeof(uint32_t));
        a->v = zalloc(nvars, sizeof(double));
        a->inv_v = zalloc(nvars, sizeof(double));
        return a;
}

/* approx.c:72-92: the instance plus a shadow over a permuted copy. */
or_approx_t * or_approx_make(or_matrix_t * m, size_t nrhs, const double * rhs,
                             const double * weight, size_t nvars,
                             const double * linear, const double * lower,
                             const double * upper)
{
        or_approx_t * a = approx_make_1(m, nrhs, rhs, weight, nvars, linear,
                                        lower, upper);
        or_matrix_t * pm = or_matrix_make(m->ncols, m->nrows, m->nnz,
                                          m->rows, m->cols, m->vals, 1);
        a->permuted = approx_make_1(pm, nrhs, rhs, weight, nvars, linear,
                                    lower, upper);
        a->permuted->owns_matrix = 1;
        or_approx_update(a);
        return a;
}

static void approx_free_1(or_approx_t * a)
{
        free(a->rhs);
        free(a->weight);
        free(a->linear);
        free(a->lower);
        free(a->upper);
        free(a->beta);
        free(a->v);
        free(a->inv_v);
        if (a->owns_matrix)
                or_matrix_free(a->matrix);
        free(a);
}

void or_approx_free(or_approx_t * a)
{
        if (a == NULL)
                return;
        if (a->permuted)
                approx_free_1(a->permuted);
        approx_free_1(a);
}

double * or_approx_vec(or_approx_t * a, int which)
{
        switch (which) {
        case 0: return a->rhs;
        case 1: return a->weight;
        case 2: return a->linear;
        case 3: return a->lower;
        default: return a->upper;
        }
}

/* approx.c:135-186: beta_i = nonzeros in row i; v_j += w_i beta_i A_ij^2
 * in the (Z-order) COO order; inv_v = 1/v, or 1 where v = 0 and c = 0. */
static void update_step_size(or_approx_t * a)
{
        or_matrix_t * m = a->matrix;
        memset(a->beta, 0, a->nrhs * sizeof(uint32_t));
        memset(a->v, 0, a->nvars * sizeof(double));
        for (size_t i = 0; i < m->nnz; i++)
                a->beta[m->rows[i]]++;
        for (size_t i = 0; i < m->nnz; i++) {
                uint32_t row = m->rows[i];
                double value = m->vals[i];
                double w = a->weight[row];
                a->v[m->cols[i]] += w * a->beta[row] * value * value;
        }
        for (size_t i = 0; i < a->nvars; i++) {
                double vi = a->v[i];
                if ((vi == 0) && (a->linear[i] == 0))
                        a->inv_v[i] = 1;
                else
                        a->inv_v[i] = 1.0 / vi;
        }
}

static void permute_fwd(const perm_t * p, double * dest, const double * src)
{
        for (size_t i = 0; i < p->n; i++)
                dest[i] = src[p->idx[i]];
}

static void permute_inv(const perm_t * p, double * dest, const double * src)
{
        for (size_t i = 0; i < p->n; i++)
                dest[i] = src[p->ridx[i]];
}

/* approx.c:188-216 */
int or_approx_update(or_approx_t * a)
{
        update_step_size(a);
        if (a->permuted) {
                or_approx_t * p = a->permuted;
                or_matrix_t * pm = p->matrix;
                permute_fwd(&pm->rperm, p->rhs, a->rhs);
                permute_fwd(&pm->rperm, p->weight, a->weight);
                permute_fwd(&pm->cperm, p->linear, a->linear);
                permute_fwd(&pm->cperm, p->lower, a->lower);
                permute_fwd(&pm->cperm, p->upper, a->upper);
                update_step_size(p);
        }
        return 0;
}

void or_approx_internals(or_approx_t * a, int permuted, uint32_t * beta,
                         double * v, double * inv_v, double * rhs,
                         double * weight, double * linear, double * lower,
                         double * upper)
{
        or_approx_t * s = permuted ? a->permuted : a;
        memcpy(beta, s->beta, s->nrhs * sizeof(uint32_t));
        memcpy(v, s->v, s->nvars * sizeof(double));
        memcpy(inv_v, s->inv_v, s->nvars * sizeof(double));
        memcpy(rhs, s->rhs, s->nrhs * sizeof(double));
        memcpy(weight, s->weight, s->nrhs * sizeof(double));
        memcpy(linear, s->linear, s->nvars * sizeof(double));
        memcpy(lower, s->lower, s->nvars * sizeof(double));
        memcpy(upper, s->upper, s->nvars * sizeof(double));
}

/* ------------------------------------------------------------------ */
/* Vectors with cached violation and values (vector.inc:1-62)         */
/* ------------------------------------------------------------------ */

typedef struct {
        double * x;        /* n (+ zero slop) */
        double * viol;     /* w (Ax - b), m (+ zero slop) */
        size_t n, m;
        int violp;
        double quad, value; /* NaN = not cached */
} vec_t;

static void vec_init(vec_t * v, size_t n, size_t m)
{
        v->n = n;
        v->m = m;
        v->x = zalloc(n, sizeof(double));
        v->viol = zalloc(m, sizeof(double));
        v->violp = 0;
        v->quad = v->value = nan("");
}

static void vec_free(vec_t * v)
{
        free(v->x);
        free(v->viol);
}

static void vec_copy(vec_t * dst, const vec_t * src)
{
        memcpy(dst->x, src->x, src->n * sizeof(double));
        if (src->violp) {
                memcpy(dst->viol, src->viol, src->m * sizeof(double));
                dst->violp = 1;
        } else {
                dst->violp = 0;
        }
        dst->quad = src->quad;
        dst->value = src->value;
}

static inline size_t pairs(size_t n)
{
        return (n + 1) / 2;
}

/* Per-thread partial pairs, combined in thread order. */
typedef struct {
        double a0, a1, b0, b1;
} part_t;

static double sum_parts(const part_t * p, int nt, int which)
{
        if (nt == 1)
                return which ? (p[0].b0 + p[0].b1) : (p[0].a0 + p[0].a1);
        double acc = 0;
        for (int t = 0; t < nt; t++)
                acc += which ? (p[t].b0 + p[t].b1) : (p[t].a0 + p[t].a1);
        return acc;
}

/* project, step_project.inc:11-25 */
static void project(vec_t * xv, const double * l, const double * u)
{
        for (size_t i = 0; i < 2 * pairs(xv->n); i++) {
                double lo = maxpd(l[i], xv->x[i]);
                xv->x[i] = minpd(lo, u[i]);
        }
        xv->violp = 0;
        xv->quad = xv->value = nan("");
}

/* compute_violation(_1), gradient_value.inc:15-81 */
static void compute_violation(vec_t * xv, or_approx_t * a)
{
        const blockm_t * b = &a->matrix->block;
        int nt = g_threads;
        part_t parts[256];
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
        for (int t = 0; t < nt; t++) {
                size_t lo, hi, r0, r1;
                split(b->nblocks, nt, t, 1, &lo, &hi);
                block_mult_range(b, lo, hi, xv->viol, xv->x);
                block_rows(b, lo, hi, &r0, &r1);
                double acc[2] = {0, 0};
                size_t end = 2 * pairs(r1);
                if (hi < b->nblocks)
                        end = r1;
                for (size_t i = r0; i < end; i++) {
                        double v = xv->viol[i] - a->rhs[i];
                        double s = a->weight[i] * v;
                        xv->viol[i] = s;
                        acc[i & 1] += s * v;
                }
                parts[t].a0 = acc[0];
                parts[t].a1 = acc[1];
        }
        xv->quad = .5 * sum_parts(parts, nt, 0);
        xv->violp = 1;
}

/* dot / dot_1, vector.inc:214-234 */
static double dot(const double * xp, const vec_t * yv)
{
        double acc[2] = {0, 0};
        for (size_t i = 0; i < 2 * pairs(yv->n); i++)
                acc[i & 1] += xp[i] * yv->x[i];
        return acc[0] + acc[1];
}

/* compute_value, gradient_value.inc:111-133 */
static double compute_value(or_approx_t * a, vec_t * xv)
{
        if (!isnan(xv->value))
                return xv->value;
        double linear = dot(a->linear, xv);
        if (isnan(xv->quad))
                compute_violation(xv, a);
        return xv->value = xv->quad + linear;
}

/* gradient / gradient_1, gradient_value.inc:142-181 */
static void gradient(vec_t * g, or_approx_t * a, vec_t * xv)
{
        if (!xv->violp)
                compute_violation(xv, a);
        const blockm_t * b = &a->matrix->block_t;
        int nt = g_threads;
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
        for (int t = 0; t < nt; t++) {
                size_t lo, hi, r0, r1;
                split(b->nblocks, nt, t, 1, &lo, &hi);
                block_mult_range(b, lo, hi, g->x, xv->viol);
                block_rows(b, lo, hi, &r0, &r1);
                size_t end = (hi < b->nblocks) ? r1 : 2 * pairs(r1);
                for (size_t i = r0; i < end; i++)
                        g->x[i] += a->linear[i];
        }
}

/* The fused A' pass + prox epilogue shared by gradient2_step_1
 * (step_project.inc:452-508), gradient2_long_step_1 (:179-236) and
 * gradient_long_step_1 (:320-375).  two: two right-hand sides (g0 at v0,
 * g1 at v1) or one (g1 at v1 only); long_step: return the estimate instead
 * of max |zp|. */
static double fused_step(or_approx_t * a, int two, int long_step,
                         const double * v0, const double * v1, double * g0,
                         double * g1, const double * z, double * zp,
                         double itheta, double theta2)
{
        const blockm_t * b = &a->matrix->block_t;
        const double * l = a->lower, * u = a->upper, * iv = a->inv_v,
                * vv = a->v, * lin = a->linear;
        int nt = g_threads;
        part_t parts[256];
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
        for (int t = 0; t < nt; t++) {
                size_t lo, hi, r0, r1;
                split(b->nblocks, nt, t, 1, &lo, &hi);
                if (two)
                        block_mult2_range(b, lo, hi, g0, g1, v0, v1);
                else
                        block_mult_range(b, lo, hi, g1, v1);
                block_rows(b, lo, hi, &r0, &r1);
                size_t end = (hi < b->nblocks) ? r1 : 2 * pairs(r1);
                double le[2] = {0, 0}, qe[2] = {0, 0}, mz[2] = {0, 0};
                for (size_t i = r0; i < end; i++) {
                        double li = lin[i];
                        if (two)
                                g0[i] += li;
                        double gi = g1[i] += li;
                        double step = itheta * iv[i];
                        double trial = z[i] - gi * step;
                        trial = maxpd(l[i], trial);
                        trial = minpd(u[i], trial);
                        zp[i] = trial;
                        if (long_step) {
                                double delta = trial - z[i];
                                le[i & 1] += gi * delta;
                                qe[i & 1] += delta * delta * theta2 * vv[i];
                        } else {
                                mz[i & 1] = maxpd(mz[i & 1], fabs(trial));
                        }
                }
                if (long_step) {
                        parts[t].a0 = le[0];
                        parts[t].a1 = le[1];
                        parts[t].b0 = qe[0];
                        parts[t].b1 = qe[1];
                } else {
                        parts[t].a0 = mz[0];
                        parts[t].a1 = mz[1];
                }
        }
        if (long_step) {
                if (nt == 1)
                        return (parts[0].a0 + parts[0].a1)
                                + .5 * (parts[0].b0 + parts[0].b1);
                double acc = 0;
                for (int t = 0; t < nt; t++)
                        acc += (parts[t].a0 + parts[t].a1)
                                + .5 * (parts[t].b0 + parts[t].b1);
                return acc;
        }
        double mx = 0;
        for (int t = 0; t < nt; t++)
                mx = fmax(mx, (parts[t].a0 > parts[t].a1) ? parts[t].a0
                                                            : parts[t].a1);
        return mx;
}

static void invalidate(vec_t * v)
{
        v->violp = 0;
        v->value = v->quad = nan("");
}

/* step / step_1, step_project.inc:34-94 */
static void step(vec_t * zp, double theta, const vec_t * g, const vec_t * z,
                 or_approx_t * a)
{
        double itheta = (1 - 1e-6) / theta;
        for (size_t i = 0; i < 2 * pairs(zp->n); i++) {
                double s = itheta * a->inv_v[i];
                double trial = z->x[i] - g->x[i] * s;
                trial = maxpd(a->lower[i], trial);
                trial = minpd(a->upper[i], trial);
                zp->x[i] = trial;
        }
        invalidate(zp);
}

/* linterp_xy(_1), vector.inc:249-335 */
static void linterp_xy(vec_t * y, vec_t * x, const vec_t * z, double theta,
                       double next_theta)
{
        double scale = 1 - theta, next_scale = 1 - next_theta;
        for (size_t i = 0; i < 2 * pairs(x->n); i++)
                x->x[i] = scale * x->x[i] + theta * z->x[i];
        for (size_t i = 0; i < 2 * pairs(x->m); i++) {
                double xv = scale * x->viol[i] + theta * z->viol[i];
                y->viol[i] = next_scale * xv + next_theta * z->viol[i];
                x->viol[i] = xv;
        }
        y->value = x->value = nan("");
        y->quad = x->quad = nan("");
}

/* dot_diff, approx.c:227-256 */
static double dot_diff(const vec_t * g, const vec_t * z, const vec_t * zp)
{
        double acc[2] = {0, 0};
        for (size_t i = 0; i < 2 * pairs(g->n); i++)
                acc[i & 1] += g->x[i] * (zp->x[i] - z->x[i]);
        return acc[0] + acc[1];
}

/* project_gradient_norm, approx.c:258-278 */
static double pg_norm(const vec_t * g, const vec_t * x, const double * l,
                      const double * u)
{
        double acc[2] = {0, 0};
        for (size_t i = 0; i < 2 * pairs(g->n); i++) {
                double xi = x->x[i];
                double xp = xi - g->x[i];
                xp = maxpd(l[i], xp);
                xp = minpd(u[i], xp);
                double d = xi - xp;
                acc[i & 1] += d * d;
        }
        return sqrt(acc[0] + acc[1]);
}

/* diff / norm_2, approx.c:480-502 */
static double diff(const double * x, const double * y, size_t n)
{
        double acc[2] = {0, 0};
        for (size_t i = 0; i < 2 * pairs(n); i++) {
                double d = x[i] - y[i];
                acc[i & 1] += d * d;
        }
        return sqrt(acc[0] + acc[1]);
}

static double norm2v(const vec_t * v)
{
        double acc[2] = {0, 0};
        for (size_t i = 0; i < 2 * pairs(v->n); i++)
                acc[i & 1] += v->x[i] * v->x[i];
        return sqrt(acc[0] + acc[1]);
}

/* struct approx_state, approx.c:280-324 */
typedef struct {
        vec_t y, z, zp, x;
        size_t iteration;
        double theta;
        vec_t g, g2, u;
        double step_length;
} state_t;

static void state_init(state_t * s, size_t n, size_t m)
{
        vec_init(&s->y, n, m);
        vec_init(&s->z, n, m);
        vec_init(&s->zp, n, m);
        vec_init(&s->x, n, m);
        s->iteration = 0;
        s->theta = 1;
        vec_init(&s->g, n, m);
        vec_init(&s->g2, n, m);
        vec_init(&s->u, n, m);
        s->step_length = 1;
}

static void state_free(state_t * s)
{
        vec_free(&s->y);
        vec_free(&s->z);
        vec_free(&s->zp);
        vec_free(&s->x);
        vec_free(&s->g);
        vec_free(&s->g2);
        vec_free(&s->u);
}

/* next_theta, approx.c:328-339 (default: theta = 2/(k+2)) */
static double next_theta(state_t * s)
{
        size_t k = ++s->iteration;
        return s->theta = 2.0 / (k + 2);
}

static void ensure_violation(vec_t * v, or_approx_t * a)
{
        if (!v->violp)
                compute_violation(v, a);
}

/* try_long_step, approx.c:343-392 */
static int try_long_step(or_approx_t * a, state_t * s, double step_length,
                         int compute_zg)
{
        int safe = (step_length <= 1 + 1e-6);
        if (safe)
                step_length = 1;
        double itheta = (step_length - 1e-6) / s->theta;
        double theta2 = s->theta / step_length;
        double expected;
        if (compute_zg) {
                ensure_violation(&s->z, a);
                ensure_violation(&s->y, a);
                expected = fused_step(a, 1, 1, s->z.viol, s->y.viol, s->g.x,
                                      s->g2.x, s->z.x, s->zp.x, itheta,
                                      theta2);
        } else {
                ensure_violation(&s->y, a);
                expected = fused_step(a, 0, 1, NULL, s->y.viol, NULL,
                                      s->g2.x, s->z.x, s->zp.x, itheta,
                                      theta2);
        }
        invalidate(&s->zp);
        double initial = compute_value(a, &s->z);
        double now = compute_value(a, &s->zp);
        if (now <= initial + expected) {
                s->step_length = step_length * 1.01;
                return 1;
        }
        s->step_length = .9 * step_length;
        if (!safe)
                step(&s->zp, s->theta, &s->g2, &s->z, a);
        return 0;
}

/* short_step, approx.c:394-415 */
static int short_step(or_approx_t * a, state_t * s, double step_length)
{
        ensure_violation(&s->z, a);
        ensure_violation(&s->y, a);
        double itheta = (1 - 1e-6) / s->theta;
        fused_step(a, 1, 0, s->z.viol, s->y.viol, s->g.x, s->g2.x, s->z.x,
                   s->zp.x, itheta, 0);
        invalidate(&s->zp);
        s->step_length = step_length * 1.01;
        if (s->step_length > 1)
                s->step_length = 1 + 1e-6;
        return 0;
}

/* iter, approx.c:417-478 */
static const vec_t * iter(or_approx_t * a, state_t * s, double * out_pg)
{
        int descent, got_gradient;
        double step_length = s->step_length;
        if (step_length <= 1) {
                descent = short_step(a, s, step_length);
                got_gradient = 1;
        } else {
                got_gradient = (out_pg != NULL)
                        || (step_length <= 1 + 1e-6);
                descent = try_long_step(a, s, step_length, got_gradient);
        }
        if (out_pg != NULL)
                *out_pg = pg_norm(&s->g, &s->z, a->lower, a->upper);
        if (!descent) {
                if (!got_gradient)
                        gradient(&s->g, a, &s->z);
                if (dot_diff(&s->g, &s->z, &s->zp) > 0) {
                        vec_copy(&s->x, &s->z);
                        vec_copy(&s->y, &s->z);
                        s->iteration = 0;
                        s->theta = 1;
                        return &s->x;
                }
        }
        if (!s->zp.violp)
                compute_violation(&s->zp, a);
        double theta = s->theta;
        double next = next_theta(s);
        linterp_xy(&s->y, &s->x, &s->zp, theta, next);
        vec_t tmp = s->z;
        s->z = s->zp;
        s->zp = tmp;
        return &s->zp;
}

/* print_log, approx.c:504-515 */
static void print_log(FILE * log, size_t k, double value, double ng,
                      double pg, double stepl, double d)
{
        if (log == NULL)
                return;
        if (d < HUGE_VAL)
                fprintf(log, "\t%10zu %12g %12g %12g %8g %12g\n", k, value,
                        ng, pg, stepl, d);
        else
                fprintf(log, "\t%10zu %12g %12g %12g %8g\n", k, value, ng,
                        pg, stepl);
}

static int approx_solve_log(or_approx_t * a, double * x, size_t niter,
                            double max_pg, double max_value,
                            double min_delta, FILE * log, size_t period,
                            double * diag, double offset, double * trace,
                            size_t trace_cap)
{
        if (a->permuted)
                a = a->permuted;
        size_t n = a->nvars;
        const perm_t * cperm = &a->matrix->cperm;
        state_t s;
        state_init(&s, a->nvars, a->nrhs);
        permute_fwd(cperm, s.x.x, x);
        project(&s.x, a->lower, a->upper);
        compute_violation(&s.x, a);
        compute_value(a, &s.x);
        vec_copy(&s.z, &s.x);
        vec_copy(&s.y, &s.x);
        double * prev_x = zalloc(n, sizeof(double));
        memcpy(prev_x, s.x.x, n * sizeof(double));

        const vec_t * center = &s.x;
        double value = compute_value(a, (vec_t *)center) + offset;
        double ng = HUGE_VAL, pg = HUGE_VAL, delta = HUGE_VAL;
        size_t i;
        int restart = 0, reason = 0;
        for (i = 0; i < niter; i++) {
                delta = HUGE_VAL;
                pg = HUGE_VAL;
                double * pgp = ((i == 0) || ((i + 1) % 10 == 0)) ? &pg : NULL;
                center = iter(a, &s, pgp);
                int restarted = (center == &s.x);
                if (restarted) {
                        if (!restart) {
                                restart = 1;
                                if (log != NULL)
                                        fprintf(log, "\t\t ");
                        }
                        if (log != NULL)
                                fprintf(log, "R");
                }
                value = compute_value(a, (vec_t *)center) + offset;
                if (trace != NULL && i < trace_cap) {
                        double * rec = trace + 6 * i;
                        rec[0] = value;
                        rec[1] = pg;
                        rec[2] = s.step_length;
                        rec[3] = s.theta;
                        rec[4] = restarted;
                        rec[5] = (double)i;
                }
                if (value < max_value) {
                        reason = 1;
                        break;
                }
                if (pg < max_pg) {
                        reason = 2;
                        break;
                }
                if ((i + 1) % 100 == 0) {
                        center = &s.x;
                        compute_violation(&s.x, a);
                        value = compute_value(a, &s.x) + offset;
                        gradient(&s.g, a, &s.x);
                        pg = pg_norm(&s.g, &s.x, a->lower, a->upper);
                        delta = diff(prev_x, s.x.x, n) / (norm2v(&s.x) + 1e-10);
                        if (value < max_value) {
                                reason = 1;
                                break;
                        }
                        if (pg < max_pg) {
                                reason = 2;
                                break;
                        }
                        if (delta < min_delta) {
                                reason = 3;
                                break;
                        }
                        memcpy(prev_x, s.x.x, n * sizeof(double));
                }
                if ((i == 0) || (period && ((i + 1) % period == 0))) {
                        restart = 0;
                        ng = norm2v(&s.g);
                        print_log(log, i + 1, value, ng, pg, s.step_length,
                                  delta);
                }
        }
        delta = diff(prev_x, center->x, n) / (norm2v(center) + 1e-10);
        value = compute_value(a, (vec_t *)center) + offset;
        gradient(&s.g, a, (vec_t *)center);
        ng = norm2v(&s.g);
        pg = pg_norm(&s.g, center, a->lower, a->upper);
        print_log(log, i + 1, value, ng, pg, s.step_length, delta);
        permute_inv(cperm, x, center->x);
        if (diag != NULL) {
                diag[0] = value;
                diag[1] = ng;
                diag[2] = pg;
                diag[3] = delta;
                diag[4] = (double)(i + 1);
        }
        free(prev_x);
        state_free(&s);
        return reason;
}

/* approx_solve, approx.c:576-708.  (The reference also writes a bare
 * newline to stdout after restart markers, approx.c:669,678; the oracle
 * does not.) */
int or_approx_solve(or_approx_t * a, double * x, size_t niter, double max_pg,
                    double max_value, double min_delta, const char * log_path,
                    size_t period, double * diag, double offset,
                    double * trace, size_t trace_cap)
{
        FILE * log = log_path ? fopen(log_path, "w") : NULL;
        int r = approx_solve_log(a, x, niter, max_pg, max_value, min_delta,
                                 log, period, diag, offset, trace, trace_cap);
        if (log)
                fclose(log);
        return r;
}

/* spg_iter, mpg.inc:155-199 */
static int spg_iter(or_approx_t * a, state_t * s, double * out_pg)
{
        size_t n = a->nvars;
        project(&s->x, a->lower, a->upper);
        gradient(&s->g, a, &s->x);
        if (out_pg != NULL)
                *out_pg = pg_norm(&s->g, &s->x, a->lower, a->upper);
        for (size_t i = 0; i < n; i++) {
                s->y.x[i] = s->x.x[i] - s->z.x[i];
                s->u.x[i] = s->g.x[i] - s->g2.x[i];
        }
        double stepl = dot(s->y.x, &s->y) / dot(s->y.x, &s->u);
        if (isnan(stepl))
                stepl = 1;
        if (stepl > 1e8)
                return 1;
        for (size_t i = 0; i < n; i++)
                s->z.x[i] = s->x.x[i] - stepl * s->g.x[i];
        project(&s->z, a->lower, a->upper);
        vec_t t = s->z;
        s->z = s->x;
        s->x = t;
        t = s->g2;
        s->g2 = s->g;
        s->g = t;
        return 0;
}

/* mpg_solve, approx.c:517-573 */
int or_mpg_solve(or_approx_t * a, double * x, size_t niter, double max_pg,
                 double max_value, double min_delta, const char * log_path,
                 size_t period, double * diag, double offset)
{
        (void)min_delta;
        FILE * log = log_path ? fopen(log_path, "w") : NULL;
        if (a->permuted)
                a = a->permuted;
        const perm_t * cperm = &a->matrix->cperm;
        state_t s;
        state_init(&s, a->nvars, a->nrhs);
        permute_fwd(cperm, s.x.x, x);
        project(&s.x, a->lower, a->upper);
        vec_copy(&s.z, &s.x);
        gradient(&s.g, a, &s.x);
        vec_copy(&s.g2, &s.g);
        int reason = 0;
        size_t i;
        for (i = 0; (i < niter) && !reason; i++) {
                double pg;
                spg_iter(a, &s, &pg);
                double value = offset + compute_value(a, &s.x);
                if (pg < max_pg)
                        reason = 2;
                if (value < max_value)
                        reason = 1;
                if (log && ((period && (i % period == 0)) || (i == 0)
                            || reason))
                        fprintf(log, "%10zu: %12g %12g\n", i + 1, pg, value);
        }
        permute_inv(cperm, x, s.x.x);
        if (diag != NULL) {
                gradient(&s.g, a, &s.x);
                diag[0] = offset + compute_value(a, &s.x);
                diag[1] = norm2v(&s.g);
                diag[2] = pg_norm(&s.g, &s.x, a->lower, a->upper);
                diag[3] = HUGE_VAL;
                diag[4] = (double)(i + 1);
        }
        state_free(&s);
        if (log)
                fclose(log);
        return 2;
}

/* ------------------------------------------------------------------ */
/* ALM (alm.c:8-322)                                                   */
/* ------------------------------------------------------------------ */

struct or_alm {
        size_t nrhs, nvars;
        or_matrix_t * matrix;
        double * linear;
        or_approx_t * approx;
        double * lambda_lower, * lambda_upper;
};

or_alm_t * or_alm_make(or_matrix_t * m, size_t nrhs, const double * rhs,
                       size_t nvars, const double * linear,
                       const double * lower, const double * upper,
                       const double * lambda_lower,
                       const double * lambda_upper)
{
        or_alm_t * alm = calloc(1, sizeof(*alm));
        alm->nrhs = nrhs;
        alm->nvars = nvars;
        alm->matrix = m;
        alm->linear = dup_or(linear, nvars, 0);
        alm->approx = or_approx_make(m, nrhs, rhs, NULL, nvars, NULL, lower,
                                     upper);
        alm->lambda_lower = dup_or(lambda_lower, nrhs, -HUGE_VAL);
        alm->lambda_upper = dup_or(lambda_upper, nrhs, HUGE_VAL);
        return alm;
}

void or_alm_free(or_alm_t * alm)
{
        if (alm == NULL)
                return;
        free(alm->linear);
        free(alm->lambda_lower);
        free(alm->lambda_upper);
        or_approx_free(alm->approx);
        free(alm);
}

or_approx_t * or_alm_approx(or_alm_t * alm)
{
        return alm->approx;
}

static double sdot(const double * x, const double * y, size_t n)
{
        double acc = 0;
        for (size_t i = 0; i < n; i++)
                acc += x[i] * y[i];
        return acc;
}

static double snorm2(const double * x, size_t n)
{
        double acc = 0;
        for (size_t i = 0; i < n; i++)
                acc += x[i] * x[i];
        return sqrt(acc);
}

static double snorm1(const double * x, size_t n)
{
        double acc = 0;
        for (size_t i = 0; i < n; i++)
                acc += fabs(x[i]);
        return acc;
}

static double snorm_inf(const double * x, size_t n, size_t * out_i)
{
        double max = -HUGE_VAL;
        size_t idx = (size_t)-1;
        for (size_t i = 0; i < n; i++) {
                double xi = fabs(x[i]);
                if (xi > max) {
                        max = xi;
                        idx = i;
                }
        }
        if (out_i)
                *out_i = idx;
        return max;
}

static void project_multipliers(double * lam, or_alm_t * alm)
{
        for (size_t i = 0; i < alm->nrhs; i++)
                lam[i] = fmax(alm->lambda_lower[i],
                              fmin(lam[i], alm->lambda_upper[i]));
}

typedef struct {
        double * violation;
        double prev_viol_norm;
        double precision;
} alm_state_t;

static int alm_iter(alm_state_t * st, or_alm_t * alm, double * x,
                    double * lam, FILE * log, size_t k, double * out_pg,
                    double * out_max_viol, size_t inner_budget,
                    size_t * inner_used)
{
        size_t nvars = alm->nvars, nrhs = alm->nrhs;
        or_approx_t * a = alm->approx;
        /* penalise_linear, alm.c:106-119 */
        or_multiply(a->linear, alm->matrix, lam, 1);
        for (size_t i = 0; i < nvars; i++)
                a->linear[i] = alm->linear[i] - a->linear[i];
        double offset = sdot(lam, a->rhs, nrhs);
        double diag[5];
        or_approx_update(a);
        size_t niter = (size_t)4294967295u; /* -1u, alm.c:255 */
        if (inner_budget != (size_t)-1) {
                size_t left = (*inner_used < inner_budget)
                        ? inner_budget - *inner_used : 0;
                if (niter > left)
                        niter = left;
        }
        int reason = approx_solve_log(a, x, niter, fmin(1, st->precision),
                                      -HUGE_VAL, 1e-11, log, 10000, diag,
                                      offset, NULL, 0);
        *inner_used += (reason == 0) ? niter : (size_t)diag[4];
        /* violation, alm.c:121-132 */
        or_multiply(st->violation, alm->matrix, x, 0);
        for (size_t i = 0; i < nrhs; i++)
                st->violation[i] -= a->rhs[i];
        double max_viol = snorm_inf(st->violation, nrhs, NULL);
        if (log != NULL)
                fprintf(log, "%4zu: %12g %12g %12g %.18g %.18g", k, max_viol,
                        snorm2(st->violation, nrhs), diag[2], diag[0],
                        sdot(x, alm->linear, nvars));
        if (out_pg)
                *out_pg = diag[2];
        if (out_max_viol)
                *out_max_viol = max_viol;
        /* update_multipliers, alm.c:182-192 */
        for (size_t i = 0; i < nrhs; i++)
                lam[i] -= a->weight[i] * st->violation[i];
        project_multipliers(lam, alm);
        /* update_precision, alm.c:235-245 */
#define UPDATE_PRECISION()                                                   \
        do {                                                                 \
                double viol = snorm_inf(st->violation, nrhs, NULL);          \
                double w = nrhs / snorm1(a->weight, nrhs);                   \
                st->precision = fmin(st->precision,                          \
                                     fmin(pow(viol, 1), pow(w, 1.5)));       \
                st->precision = fmax(st->precision, 1e-7);                   \
        } while (0)
        if (reason != 2) {
                if (log != NULL)
                        fprintf(log, " -stalled-\n");
                UPDATE_PRECISION();
                return 1;
        }
        /* update_weights, alm.c:194-212 */
        {
                double norm = snorm2(st->violation, nrhs);
                if (!(norm < .5 * st->prev_viol_norm)) {
                        double scale = 2 * fmin(1, norm / st->prev_viol_norm);
                        for (size_t i = 0; i < nrhs; i++)
                                a->weight[i] *= scale;
                        size_t max_i;
                        double max = snorm_inf(st->violation, nrhs, &max_i);
                        if (max > .5 * norm)
                                a->weight[max_i] *= 10;
                }
                st->prev_viol_norm = norm;
        }
        UPDATE_PRECISION();
#undef UPDATE_PRECISION
        if (log != NULL)
                fprintf(log, " (%8g)\n", snorm1(a->weight, nrhs) / nrhs);
        return 0;
}

/* alm_solve, alm.c:289-322 */
int or_alm_solve(or_alm_t * alm, size_t niter, double * x, double * lambda,
                 const char * log_path, double * diag, size_t inner_budget,
                 size_t * inner_used)
{
        FILE * log = log_path ? fopen(log_path, "w") : NULL;
        alm_state_t st;
        st.violation = calloc(alm->nrhs ? alm->nrhs : 1, sizeof(double));
        st.prev_viol_norm = HUGE_VAL;
        st.precision = 1;
        project_multipliers(lambda, alm);
        size_t used = 0;
        double pg = HUGE_VAL, max_viol = HUGE_VAL;
        int ret = 1;
        for (size_t i = 0; i < niter; i++) {
                int status = alm_iter(&st, alm, x, lambda, log, i + 1, &pg,
                                      &max_viol, inner_budget, &used);
                if ((max_viol < 1e-5) && (status || (pg < 1e-5))) {
                        ret = 0;
                        break;
                }
                /* the inner budget is a harness stop, not the reference's */
                if (inner_budget != (size_t)-1 && used >= inner_budget)
                        break;
        }
        if (diag != NULL) {
                diag[0] = sdot(x, alm->linear, alm->nvars);
                diag[1] = max_viol;
                diag[2] = pg;
        }
        if (inner_used)
                *inner_used = used;
        free(st.violation);
        if (log)
                fclose(log);
        return ret;
}

/* ------------------------------------------------------------------ */
/* Single fused epilogues, for kernel-by-kernel checks                 */
/* ------------------------------------------------------------------ */

static or_approx_t * pick(or_approx_t * a, int permuted)
{
        return (permuted && a->permuted) ? a->permuted : a;
}

double or_k_violation(or_approx_t * a, int permuted, const double * x,
                      double * viol)
{
        a = pick(a, permuted);
        vec_t v;
        vec_init(&v, a->nvars, a->nrhs);
        memcpy(v.x, x, a->nvars * sizeof(double));
        compute_violation(&v, a);
        memcpy(viol, v.viol, a->nrhs * sizeof(double));
        double q = v.quad;
        vec_free(&v);
        return q;
}

void or_k_gradient(or_approx_t * a, int permuted, const double * viol,
                   double * g)
{
        a = pick(a, permuted);
        vec_t v, gv;
        vec_init(&v, a->nvars, a->nrhs);
        vec_init(&gv, a->nvars, a->nrhs);
        memcpy(v.viol, viol, a->nrhs * sizeof(double));
        v.violp = 1;
        gradient(&gv, a, &v);
        memcpy(g, gv.x, a->nvars * sizeof(double));
        vec_free(&v);
        vec_free(&gv);
}

static double * padded(const double * src, size_t n)
{
        double * p = zalloc(n, sizeof(double));
        if (src)
                memcpy(p, src, n * sizeof(double));
        return p;
}

double or_k_gradient2_step(or_approx_t * a, int permuted, const double * v0,
                           const double * v1, const double * z, double theta,
                           double * g0, double * g1, double * zp)
{
        a = pick(a, permuted);
        size_t n = a->nvars, m = a->nrhs;
        double * pv0 = padded(v0, m), * pv1 = padded(v1, m),
                * pz = padded(z, n), * pg0 = padded(NULL, n),
                * pg1 = padded(NULL, n), * pzp = padded(NULL, n);
        double r = fused_step(a, 1, 0, pv0, pv1, pg0, pg1, pz, pzp,
                              (1 - 1e-6) / theta, 0);
        memcpy(g0, pg0, n * sizeof(double));
        memcpy(g1, pg1, n * sizeof(double));
        memcpy(zp, pzp, n * sizeof(double));
        free(pv0); free(pv1); free(pz); free(pg0); free(pg1); free(pzp);
        return r;
}

double or_k_gradient_long_step(or_approx_t * a, int permuted, int two,
                               const double * v0, const double * v1,
                               const double * z, double theta, double length,
                               double * g0, double * g1, double * zp)
{
        a = pick(a, permuted);
        size_t n = a->nvars, m = a->nrhs;
        double * pv0 = padded(v0, m), * pv1 = padded(v1, m),
                * pz = padded(z, n), * pg0 = padded(NULL, n),
                * pg1 = padded(NULL, n), * pzp = padded(NULL, n);
        double r = fused_step(a, two, 1, two ? pv0 : NULL, pv1,
                              two ? pg0 : NULL, pg1, pz, pzp,
                              (length - 1e-6) / theta, theta / length);
        if (two && g0)
                memcpy(g0, pg0, n * sizeof(double));
        memcpy(g1, pg1, n * sizeof(double));
        memcpy(zp, pzp, n * sizeof(double));
        free(pv0); free(pv1); free(pz); free(pg0); free(pg1); free(pzp);
        return r;
}

void or_k_linterp_xy(size_t n, size_t m, double * y_viol, double * x,
                     double * x_viol, const double * z, const double * z_viol,
                     double theta, double next_theta)
{
        vec_t y, xv, zv;
        vec_init(&y, n, m);
        vec_init(&xv, n, m);
        vec_init(&zv, n, m);
        memcpy(xv.x, x, n * sizeof(double));
        memcpy(xv.viol, x_viol, m * sizeof(double));
        memcpy(zv.x, z, n * sizeof(double));
        memcpy(zv.viol, z_viol, m * sizeof(double));
        linterp_xy(&y, &xv, &zv, theta, next_theta);
        memcpy(y_viol, y.viol, m * sizeof(double));
        memcpy(x, xv.x, n * sizeof(double));
        memcpy(x_viol, xv.viol, m * sizeof(double));
        vec_free(&y);
        vec_free(&xv);
        vec_free(&zv);
}

double or_k_project_gradient_norm(or_approx_t * a, int permuted,
                                  const double * g, const double * x)
{
        a = pick(a, permuted);
        vec_t gv, xv;
        vec_init(&gv, a->nvars, 0);
        vec_init(&xv, a->nvars, 0);
        memcpy(gv.x, g, a->nvars * sizeof(double));
        memcpy(xv.x, x, a->nvars * sizeof(double));
        double r = pg_norm(&gv, &xv, a->lower, a->upper);
        vec_free(&gv);
        vec_free(&xv);
        return r;
}

double or_k_dot_diff(size_t n, const double * g, const double * z,
                     const double * zp)
{
        vec_t gv, zv, zpv;
        vec_init(&gv, n, 0);
        vec_init(&zv, n, 0);
        vec_init(&zpv, n, 0);
        memcpy(gv.x, g, n * sizeof(double));
        memcpy(zv.x, z, n * sizeof(double));
        memcpy(zpv.x, zp, n * sizeof(double));
        double r = dot_diff(&gv, &zv, &zpv);
        vec_free(&gv);
        vec_free(&zv);
        vec_free(&zpv);
        return r;
}
