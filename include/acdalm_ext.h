/* libacdalm extensions: device control, error reporting, precision modes,
 * device-resident SpMV, solve statistics.  None of these has a counterpart
 * in the reference; legacy callers never need them.
 *
 * Error convention: the drop-in entry points keep the reference's return
 * values on success; device failures come back as the negative codes below
 * (never as 0/1/2/3), and acdalm_last_error() describes the last one.
 */
#ifndef ACDALM_EXT_H
#define ACDALM_EXT_H
#include <stddef.h>
#include <stdio.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define ACDALM_OK 0
#define ACDALM_ECUDA (-1)      /* a CUDA call failed */
#define ACDALM_ETIMEOUT (-2)   /* a device-side wait gave up */
#define ACDALM_ENOMEM (-3)     /* device or host allocation failed */
#define ACDALM_EINVAL (-4)     /* bad argument (sizes, pointers, modes) */
#define ACDALM_ENONFINITE (-5) /* the iterates stopped being finite */
#define ACDALM_ENODEV (-6)     /* no usable CUDA device */
#define ACDALM_ETIMELIMIT (-7) /* the solve ran past its time limit
                                  (ACDALM_SOLVE_TIMEOUT seconds, default 900) */

struct sparse_matrix;
struct approx;
struct alm;

/* Message for the calling thread's last error ("" if none). */
const char * acdalm_last_error(void);
/* Kernels the library has launched so far (all threads). */
unsigned long long acdalm_launch_count(void);
/* Code of the calling thread's last error (0 if none); clears it. */
int acdalm_take_error(void);

/* ---- SpMV on the device ---- */
#define ACDALM_SPMV_SELL 0  /* warp-sliced ELL, one warp per slice (default) */
#define ACDALM_SPMV_BLOCK 1 /* the 4-row block arena of the reference */
#define ACDALM_SPMV_CSR 2   /* CSR, a sub-warp per row */
/* SELL with fused multiply-adds and a lane tree per row: not bit-identical
 * to the reference (within 1e-12 relative), but not bound by the FP64
 * issue rate the separately rounded product needs. */
#define ACDALM_SPMV_SELL_FMA 3
/* Variant used by sparse_matrix_multiply{,_2}; returns the previous one. */
int acdalm_spmv_variant(int variant);
/* y = op(A) x with x and y already in device memory, launched on `stream`
 * (a cudaStream_t, NULL = default stream), FP64.  The layout is uploaded on
 * first use.  Returns 0 or a negative code. */
int acdalm_spmv_device(const struct sparse_matrix * a, int variant,
                       int transpose, const double * x, double * y,
                       void * stream);
/* Same in FP32 (values rounded to float once, at upload). */
int acdalm_spmv_device_f32(const struct sparse_matrix * a, int variant,
                           int transpose, const float * x, float * y,
                           void * stream);
/* Bytes of device memory the matrix's uploaded layouts occupy. */
size_t acdalm_matrix_device_bytes(const struct sparse_matrix * a);

/* ---- solver controls ---- */
#define ACDALM_PRECISION_FP64 0  /* everything in FP64 (the default) */
#define ACDALM_PRECISION_MIXED 1 /* FP32 inner iterations, FP64 outer loop
                                    and final refinement */
#define ACDALM_PRECISION_AUTO 2  /* MIXED for an LP with at least 500,000
                                    nonzeros, FP64 below (FP32 iterations
                                    pay off on large LPs; on small ones
                                    their extra iterations cost more than
                                    they save) */
int alm_set_precision(struct alm *, int mode);
/* Stop alm_solve when the relative KKT residual (max of the primal, dual
 * and gap terms, FP64, checked after every outer iteration) is <= tol; it
 * then replaces the reference's stop rule (largest violation < 1e-5 and
 * projected gradient < 1e-5).  0 = off, the default. */
int alm_set_kkt_tolerance(struct alm *, double tol);
/* Cap on the total inner iterations of one alm_solve (0 = none). */
int alm_set_inner_budget(struct alm *, uint64_t budget);

typedef struct acdalm_stats {
        double seconds;           /* device time of the last solve */
        uint64_t inner_iterations;
        uint64_t outer_iterations;
        double rel_kkt;           /* FP64 relative KKT residual at exit */
        double primal, dual, gap; /* its three terms */
        double objective;
        int status;               /* 0 ok, or a negative ACDALM_E* code */
        int precision;            /* ACDALM_PRECISION_* used */
        uint64_t fp32_inner_iterations; /* of which ran in FP32 */
} acdalm_stats_t;
int alm_last_stats(struct alm *, acdalm_stats_t * out);
int approx_last_stats(struct approx *, acdalm_stats_t * out);

/* Autotuning of the whole-GPU solve (alm_solve): builds the instance's
 * device layout with each candidate cap on the steps of a slice (0 = the
 * plain width rule, 4, 8, 12, 16; more lanes per row for fewer steps), times
 * `iterations` APPROX iterations of the instance with each, and keeps the
 * fastest for its next solves (*chosen, may be NULL).  The choice is
 * remembered for instances of the same size class (row, column and nonzero
 * counts within half an octave), which then skip the timing.  Without it
 * the cap is ACDALM_SELL_STEPS, else 8.  No reference counterpart. */
int acdalm_autotune(struct alm *, size_t iterations, int * chosen);

/* Tracing of the whole-GPU solve (alm_solve): when count > 0, each CTA of
 * the next solves records, for the team reductions first .. first + count -
 * 1 (counted from 1 in each solve; two per steady-state inner iteration),
 * three %globaltimer stamps (ns): entering the reduction (its warp 0's part
 * of the pass done), after its block reduction (the whole CTA done), and
 * leaving it (every CTA's partials summed).  alm_trace_copy writes them as
 * out[((e - first) * ctas + cta) * 3 + phase] (cap values at most) and the
 * sizes to *ctas and *count; with out NULL it reports the sizes only.
 * count = 0 turns tracing off.  A traced solve runs a separately compiled
 * kernel (fused multiply-adds), so untraced solves pay nothing for the
 * feature.  No reference counterpart. */
int alm_set_trace(struct alm *, uint64_t first, uint64_t count);
int alm_trace_copy(struct alm *, uint64_t * out, size_t cap, size_t * ctas, size_t * count);

/* Rounding of the solver kernels: 0 (default) fused multiply-adds; 1 the
 * reference's separate rounding of every product and sum, which makes the
 * per-element results of each pass bit-identical to the reference's (the
 * reductions still sum in a different order).  Returns the previous value. */
int acdalm_set_rounding(int exact);

/* cudaStream_t the instance launches on (created with the instance). */
void * alm_stream(struct alm *);
void * approx_stream(struct approx *);


/* ---- batches: many independent LPs at once ---- */
/* A batch borrows alm_t instances (made with alm_make, settings from
 * alm_set_*).  acdalm_batch_solve runs alm_solve on every instance in one
 * persistent launch: each LP runs on its own CTA, whose barriers are CTA
 * barriers; CTAs take LPs from a shared counter, largest first, until all
 * are done.  x[i] and lambda[i] are instance i's host arrays (in/out, as in
 * alm_solve); ret[i] (may be NULL) its alm_solve return value; diag (may be
 * NULL) 3 doubles per instance.  alm_last_stats(instances[i]) reports each
 * instance.  Returns 0, or the first negative ACDALM_E* code. */
typedef struct acdalm_batch acdalm_batch_t;
acdalm_batch_t * acdalm_batch_make(struct alm * const * instances, size_t count);
int acdalm_batch_solve(acdalm_batch_t * b, size_t niter, double * const * x,
                       double * const * lambda, int * ret, double * diag);
/* Device time of the last acdalm_batch_solve launch, seconds. */
double acdalm_batch_seconds(acdalm_batch_t * b);
int acdalm_batch_free(acdalm_batch_t * b);

/* ---- serving: continuous batching ---- */
/* A server accepts LPs at any time and solves them to a relative KKT
 * residual <= kkt_tol (alm_solve with alm_set_kkt_tolerance; precision an
 * ACDALM_PRECISION_* mode).  Builder threads (builder_threads, 0 = half
 * the cores) prepare each LP's layouts, one-CTA requests first (a larger
 * one that has waited 10 s goes next).  Each LP runs in
 * its own launch and stream, beside the others: on one CTA up to 150,000
 * nonzeros, on a thread-block cluster of 4, 8 or 16 CTAs above that, one
 * CTA per SM.  Built requests are admitted while the running solves leave
 * enough SMs free for the request's team, its device footprint fits
 * device_budget bytes (0 = 80% of the free memory) and fewer than
 * max_inflight solves run (0 = 128): one-CTA requests first in arrival
 * order, then cluster requests with the most nonzeros first; a request
 * passed over for 10 s blocks the ones behind it.  A finished solve is
 * retired and its memory returned.  The result of an LP does not depend on
 * what else runs (a fixed team, deterministic reductions). */
typedef struct acdalm_server acdalm_server_t;
acdalm_server_t * acdalm_server_create(size_t device_budget, int max_inflight,
                                       int precision, double kkt_tol,
                                       int builder_threads);
/* Copies the LP (the arguments of sparse_matrix_make + alm_make; NULL
 * vectors take alm_make's defaults) and queues it; returns its id (>= 0)
 * or a negative code. */
long long acdalm_server_submit(acdalm_server_t * s, size_t nrows, size_t ncols,
                               size_t nnz, const uint32_t * rows,
                               const uint32_t * cols, const double * values,
                               const double * rhs, const double * linear,
                               const double * lower, const double * upper,
                               const double * lambda_lower,
                               const double * lambda_upper);
/* Waits up to timeout seconds for finished requests; writes up to cap ids
 * and returns how many. */
int acdalm_server_poll(acdalm_server_t * s, long long * ids, int cap, double timeout);
/* Results of a finished request (then forgotten): x (ncols) and lambda
 * (nrows) may be NULL; st the solve's statistics (seconds = admission to
 * completion); *latency = submission to completion, seconds.  Returns the
 * request's alm_solve value or a negative code. */
int acdalm_server_result(acdalm_server_t * s, long long id, double * x,
                         double * lambda, acdalm_stats_t * st, double * latency);
/* Stops the server after the running solves finish; unfinished requests
 * are dropped. */
int acdalm_server_destroy(acdalm_server_t * s);
/* Caps each request built after the call at `budget` inner iterations in
 * all (alm_set_inner_budget); 0 = no cap, the default. */
int acdalm_server_set_inner_budget(acdalm_server_t * s, uint64_t budget);

/* ---- layout inspection (for parity checks against the reference) ---- */
/* The 4-row block arena of A (transpose = 0) or A' (1), byte for byte the
 * reference's (spmv/spmv_block.c:124-149): returns its size in bytes and
 * the block count in *nblocks. */
size_t acdalm_block_bytes(struct sparse_matrix * a, int transpose,
                          size_t * nblocks);
int acdalm_block_copy(struct sparse_matrix * a, int transpose,
                      size_t * offsets, void * arena, size_t bytes);
/* CSR of A or A' (spmv/spmv_csr.c:27-80): nrows+1 row pointers, nnz
 * columns and values. */
int acdalm_csr_copy(struct sparse_matrix * a, int transpose,
                    uint32_t * rows_indices, uint32_t * columns,
                    double * values);
/* The warp-sliced ELL ("SELL") layout the ACDALM_SPMV_SELL variant uploads
 * for A (transpose = 0) or A' (1); no reference counterpart.  Slice s holds
 * 32 / L rows from device row row0[s], L = 1 << (ptr[s] & 127) lanes per
 * row; entry k of the slice's r-th row is element (ptr[s] & ~127) +
 * 128 (k / 4L) + 4 (r L + (k / 4) % L) + k % 4 of columns / values;
 * padding entries have value 0.  Device row d is matrix row row_of_d[d].
 * With ptr NULL, stores the slice and element counts only; otherwise
 * *nslices and *nelems give the capacities of row0 (nslices), ptr
 * (nslices + 1), columns and values (nelems); row_of_d holds one entry per
 * row of the operator. */
int acdalm_sell_copy(struct sparse_matrix * a, int transpose, size_t * nslices,
                     size_t * nelems, int64_t * ptr, int32_t * row0,
                     int32_t * columns, double * values, int32_t * row_of_d);
/* Row (row = 1) or column permutation, idx = new -> old, ridx = old -> new
 * (spmv/permutation.c:63-125). */
int acdalm_perm_copy(struct sparse_matrix * a, int row, uint32_t * idx,
                     uint32_t * ridx);
/* The APPROX instance an ALM instance solves with: its approx_weight() is
 * the ALM's per-row weight vector, which persists across alm_solve calls
 * (alm.c:194-212); resetting it to 1 restarts the weighting. */
struct approx * acdalm_alm_approx(struct alm * m);
/* The permuted shadow matrix approx_make builds (approx/approx.c:84-88). */
struct sparse_matrix * acdalm_approx_permuted_matrix(struct approx * a);
/* Step sizes of the instance as the solver computes them on the device, in
 * original order: beta (nrhs), v and inv_v (nvars), approx/approx.c:135-186
 * (bit-identical to the reference's permuted instance). */
int acdalm_approx_step_sizes(struct approx * a, double * beta, double * v,
                             double * inv_v);

/* ---- layouts built on the device ---- */
/* The reference's layouts of a matrix built on the GPU from triplets
 * already in DEVICE memory (rows, cols: u32; values: f64; distinct
 * (row, column) pairs): with permute = 1 the nonzero-count permutations of
 * rows and columns (spmv/permutation.c:63-125; row_idx, col_idx: new -> old,
 * nrows and ncols entries), else the identity; and the CSR of A (ptr:
 * nrows + 1, columns and vals: nnz) and of A' (ptr_t: ncols + 1, columns_t,
 * vals_t) of the permuted matrix, ordered as spmv/spmv_csr.c:27-80 orders
 * them.  Byte for byte what sparse_matrix_make(..., permute) holds
 * (acdalm_perm_copy, acdalm_csr_copy).  All arrays are device memory; the
 * work runs on `stream` (NULL = default) and the call returns when it is
 * done.  Out-of-range triplets return ACDALM_EINVAL before anything is
 * indexed by them.  No reference counterpart. */
int acdalm_layout_device(size_t nrows, size_t ncols, size_t nnz, const uint32_t * rows,
                         const uint32_t * cols, const double * values, int permute,
                         uint32_t * row_idx, uint32_t * col_idx, uint32_t * ptr,
                         uint32_t * columns, double * vals, uint32_t * ptr_t,
                         uint32_t * columns_t, double * vals_t, void * stream);

/* ---- binary instances ---- */
/* The content of alm_read's text format (alm.h) in binary: the magic
 * "ACDALMB1", u64 nrows, ncols, nnz, then the matrix's rows, columns (u32)
 * and values (f64), rhs, linear, lower, upper, dual lower, dual upper
 * (f64), host byte order.  No reference counterpart.  Write returns 0 or
 * ACDALM_EINVAL; read returns a new instance owning a new matrix (free both
 * as after alm_read) or NULL. */
int acdalm_write_binary(struct alm * m, FILE * stream);
struct alm * acdalm_read_binary(FILE * stream);
/* An LP in free-format MPS (ROWS, COLUMNS, RHS, RANGES, BOUNDS, OBJSENSE;
 * integer markers ignored), as min c'x s.t. A x = b, l <= x <= u: every
 * inequality or ranged row r gets a slack column (coefficient -1 in row r,
 * bounded by the row's interval), appended after the file's columns in row
 * order; equality rows stay equalities; multipliers are free; OBJSENSE MAX
 * negates c.  Returns a new instance owning a new matrix, or NULL
 * (acdalm_last_error names the line). */
struct alm * acdalm_read_mps(FILE * stream);

/* ---- solving without allocating ---- */
/* approx_solve for callers that cannot call cudaMalloc when they solve:
 * frameworks whose caching allocator has already taken the device memory
 * budget, and latency-bound loops that cannot take cudaMalloc's implicit
 * device-wide synchronisation.  No counterpart in the reference.
 *
 * Same arguments and return values as approx_solve (approx.h), except: x is
 * a DEVICE array of n doubles (original order), updated in place; there is
 * no log; OUT_diagnosis (NULL or 5 doubles) is host memory; the work is
 * launched on `stream` (a cudaStream_t, NULL = the default stream) and the
 * call returns when it is done.
 *
 * It allocates nothing: all solver scratch lives in one fixed 32 MiB device
 * array inside the library, which every GPU that loads the library holds
 * until the process exits.  Instances larger than that array holds (about
 * 12 n + 6 m <= 4.17 million doubles) are rejected with ACDALM_EINVAL.  The
 * instance's own device copy (matrix layout and vectors) must already exist:
 * call approx_solve, mpg_solve or cd_solve on it once first.  The first call
 * on each device also looks up the array's device address; make that first
 * call before any stream capture.  Every call shares the one array, so
 * calls that overlap on the GPU (other threads, other streams) race. */
int approx_solve_static(double * x, size_t n, struct approx * approx,
                        size_t niter, double max_pg, double max_value,
                        double min_delta, double * OUT_diagnosis,
                        double offset, void * stream);

#ifdef __cplusplus
}
#endif
#endif
