/* Sparse matrices and sparse matrix / dense vector products.
 *
 * The entry points of the reference's spmv/spmv.h:11-84, with the same
 * argument meaning and return values.  libacdalm builds the same host
 * layouts as the reference, byte for byte (Z-order COO, CSR of A and A',
 * 4-row block arenas, nonzero-count permutations), and runs the products on
 * the GPU.
 */
#ifndef ACDALM_SPMV_H
#define ACDALM_SPMV_H
#include <stdint.h>
#include <stddef.h>
#include <stdio.h>
#include "thread_pool.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct sparse_matrix sparse_matrix_t;
/* Call once before creating a matrix (spmv.h:12-13).  Also selects and
 * initialises the CUDA device (device 0 unless ACDALM_DEVICE is set). */
void sparse_matrix_init(void);

/* A nrows x ncolumns matrix from nnz (row, column, value) triplets in any
 * order, without repeats.  permute != 0 renumbers rows and columns by
 * nonzero count within windows of 256 (spmv.h:15-24).  NULL on error. */
sparse_matrix_t * sparse_matrix_make(size_t ncolumns, size_t nrows,
                                     size_t nnz,
                                     const uint32_t * rows,
                                     const uint32_t * columns,
                                     const double * values,
                                     int permute);
/* A new matrix from the triplets of an existing one (spmv.h:25-26). */
sparse_matrix_t * sparse_matrix_copy(const sparse_matrix_t * matrix,
                                     int permute);
/* Frees host and device storage; NULL is ignored; returns 0 (:27-29). */
int sparse_matrix_free(sparse_matrix_t *);

/* Read-only accessors; the triplets come back in Z (Morton) order, as the
 * reference stores them (:31-39). */
size_t sparse_matrix_ncolumns(sparse_matrix_t *);
size_t sparse_matrix_nrows(sparse_matrix_t *);
size_t sparse_matrix_nnz(sparse_matrix_t *);
const uint32_t * sparse_matrix_rows(sparse_matrix_t *);
const uint32_t * sparse_matrix_columns(sparse_matrix_t *);
const double * sparse_matrix_values(sparse_matrix_t *);

/* dest[i] = src[idx[i]] (direction >= 0) or src[ridx[i]] (direction < 0)
 * with the row / column permutation; returns 1 if n does not match
 * (spmv.h:41-44, permutation.c:136-148). */
int sparse_matrix_row_permute(sparse_matrix_t *, double * dest, size_t n,
                              const double * src, int direction);
int sparse_matrix_col_permute(sparse_matrix_t *, double * dest, size_t n,
                              const double * src, int direction);

/* OUT_y <- op(A) x, op = identity (transpose = 0) or transpose, on the GPU.
 * ny and nx are checked against the shape.  pool is accepted and ignored.
 * Results are bit-identical to the reference's block product.  Returns 0,
 * or a negative ACDALM_E* code on a CUDA failure (spmv.h:46-62). */
int sparse_matrix_multiply(double * OUT_y, size_t ny,
                           const sparse_matrix_t * a,
                           const double * x, size_t nx,
                           int transpose,
                           thread_pool_t * pool);
/* Two right-hand sides in one pass over the matrix (spmv.h:63-74). */
int sparse_matrix_multiply_2(double ** OUT_y, size_t ny,
                             const sparse_matrix_t * a,
                             const double ** x, size_t nx,
                             int transpose,
                             thread_pool_t * pool);

/* Text format: "nrows ncolumns nnz" then nnz "row column value" triplets
 * (spmv.h:76-83).  NULL on failure. */
sparse_matrix_t * sparse_matrix_read(FILE * stream, int permute);
#ifdef __cplusplus
}
#endif
#endif
