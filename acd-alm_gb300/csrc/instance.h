// Device-resident state of one LP instance (an approx_t or alm_t) and the
// host entry points that launch the solver kernels on it.
#pragma once
#include <cuda_runtime.h>

#include <cstdio>
#include <vector>

#include "layout.h"

namespace acd {

struct LogRec;

// Every array of one instance, in device order, carved from one
// allocation.  FP64 throughout; `f32` holds the FP32 copies the mixed
// precision mode uses (allocated on first use).
struct DevInstance {
        int m = 0, n = 0;
        int64_t nnz = 0;
        cudaStream_t stream = nullptr;
        int priority = 0;  // of the stream create() makes (lower runs sooner)
        void * mem = nullptr;
        size_t bytes = 0;

        // SELL operators (FP64 values)
        int a_nslices = 0, at_nslices = 0;
        int64_t * a_ptr = nullptr, * at_ptr = nullptr;
        int32_t * a_row0 = nullptr, * at_row0 = nullptr;
        int32_t * a_col = nullptr, * at_col = nullptr;
        double * a_val = nullptr, * at_val = nullptr;
        int max_width_a = 0, max_width_at = 0;

        // permutations and constants
        int32_t * row_orig = nullptr;  // m: device row -> original row
        int32_t * col_orig = nullptr;  // n: device col -> original col
        double * beta = nullptr;       // m

        // problem vectors (m): rhs, weights, multiplier bounds, lambda, r
        double * b = nullptr, * w = nullptr, * lam_lo = nullptr,
               * lam_hi = nullptr, * lam = nullptr, * r = nullptr;
        // problem vectors (n): objective, bounds, inner linear, v, 1/v, x
        double * c0 = nullptr, * l = nullptr, * u = nullptr, * c = nullptr,
               * v = nullptr, * inv_v = nullptr, * x = nullptr;
        // workspace (n): z, zp, x, g, g2, prev, prev_alt, alt_x, u
        double * wn[9] = {};
        // workspace (2m each): violation vectors in interleaved pairs --
        // (z, y), (zp, the y its A pass writes), (x, x's spare)
        double * wm[3] = {};

        // team control, reduction slots, log ring, outputs
        void * ctl = nullptr;          // TeamCtl
        double * slots = nullptr;
        double * result = nullptr;
        LogRec * log = nullptr;
        int * log_count = nullptr;
        int log_cap = 0;
        void * out = nullptr;          // AlmOut / approx output block
        int grid_blocks = 0;           // cooperative grid size
        // phase timestamps of the last traced grid solve (alm_set_trace)
        unsigned long long * trace_rec = nullptr;
        size_t trace_cap = 0;          // records the buffer holds
        size_t trace_ctas = 0, trace_count = 0;  // of the last traced launch
        int block_threads = 256;

        // FP32 copies for the mixed precision mode (allocated on first use)
        void * mem32 = nullptr;
        size_t bytes32 = 0;
        float * a_valf = nullptr, * at_valf = nullptr;
        float * bf = nullptr, * wf = nullptr;                       // m
        float * cf = nullptr, * lf = nullptr, * uf = nullptr,       // n
              * vf = nullptr, * ivf = nullptr, * d = nullptr;
        float * wnf[9] = {};
        float * wmf[3] = {};

        int create(const DeviceLayout & lay);
        int ensure_f32(const DeviceLayout & lay);
        // Device bytes create() (+ ensure_f32 when mixed) would allocate.
        static size_t footprint(const DeviceLayout & lay, bool mixed);
        void destroy();
};

// Host-side view of the vectors an upload takes, in ORIGINAL order.
struct HostVectors {
        const double * b = nullptr;       // m
        const double * w = nullptr;       // m
        const double * lam_lo = nullptr;  // m
        const double * lam_hi = nullptr;  // m
        const double * c0 = nullptr;      // n
        const double * l = nullptr;       // n
        const double * u = nullptr;       // n
};

// Whether an LP with nnz nonzeros runs FP32 inner iterations under an
// ACDALM_PRECISION_* mode (AUTO: from kAutoMixedNnz nonzeros on).
constexpr int64_t kAutoMixedNnz = 500000;
inline bool mixed_for(int precision, int64_t nnz)
{
        return precision == 1 || (precision == 2 && nnz >= kAutoMixedNnz);
}

struct AlmSettings {
        unsigned long long inner_budget = 0;
        double kkt_tol = 0;
        int precision = 0;  // ACDALM_PRECISION_*
        // grid-team reductions first .. first + count - 1 are traced
        unsigned trace_first = 0, trace_count = 0;
};

struct SolveStats {
        double seconds = 0;
        unsigned long long inner = 0, outer = 0, inner_fp32 = 0;
        double rel_kkt = 0, primal = 0, dual = 0, gap = 0, objective = 0;
        int status = 0;
        int precision = 0;
};

// alm_solve on the device.  x (n) and lam (m) are host arrays in original
// order, updated in place; w_out (m, original order) receives the final
// weights and c_out (n) the final penalised linear term.  Returns the
// reference's 0/1 or a negative ACDALM_E* code.
int run_alm(DevInstance & d, const HostVectors & hv, size_t niter, double * x,
            double * lam, FILE * log, double * diag3, const AlmSettings & s,
            double * w_out, double * c_out, SolveStats & st,
            const DeviceLayout * lay = nullptr);

// One LP of a batch (run_alm_batch): its device instance, host vectors
// and settings, and where its results go.
struct BatchEntry {
        DevInstance * dev = nullptr;
        const DeviceLayout * lay = nullptr;
        HostVectors hv;
        AlmSettings settings;
        double * x = nullptr;
        double * lam = nullptr;
        double * diag3 = nullptr;
        double * w_out = nullptr;
        double * c_out = nullptr;
        SolveStats * stats = nullptr;
        int ret = 0;
};

// Solves every entry with one persistent launch, one LP per CTA, largest
// first.  Returns 0 or the first negative code; each entry's ret holds its
// own outcome.  *seconds receives the device time of the launch.
int run_alm_batch(std::vector<BatchEntry> & entries, size_t niter, double * seconds);

// The phase timestamps of the instance's last traced grid solve
// (AlmSettings::trace_*): ctas x count x kTracePhases values, or only the
// sizes when out is null.
int copy_trace(DevInstance & d, unsigned long long * out, size_t cap, size_t * ctas,
               size_t * count);

// One asynchronous ALM solve on one CTA (the server's unit of work): the
// launch records `done` on the instance's stream.
struct AlmLaunch {
        struct Impl;
        Impl * impl;
        cudaEvent_t done = nullptr;
        AlmLaunch();
        ~AlmLaunch();
        AlmLaunch(const AlmLaunch &) = delete;
        AlmLaunch & operator=(const AlmLaunch &) = delete;
};
// team = CTAs working on the LP: 1 (one CTA) or a thread-block cluster of
// 2..16 CTAs.
int alm_launch_async(DevInstance & d, const HostVectors & hv, size_t niter, double * x,
                     double * lam, const AlmSettings & s, const DeviceLayout * lay,
                     AlmLaunch & h, int team = 1);
// The largest cluster (CTAs) the device can run one LP's solve on (16 when
// the hardware allows it, else 8, 4, ...).
int max_cluster_team();
// After `done`: status, results (x, lambda in original order) and stats.
int alm_collect(DevInstance & d, AlmLaunch & h, double * x, double * lam, double * diag3,
                SolveStats & st);

// approx_solve on the device over the instance's uploaded vectors (b, w,
// c0 as the linear term, l, u; step sizes recomputed).  Returns the reason
// or a negative code.
int run_approx(DevInstance & d, const HostVectors & hv, double * x,
               size_t niter, double max_pg, double max_value, double min_delta,
               FILE * log, size_t period, double * diag5, double offset,
               SolveStats & st);

// mpg_solve (spectral projected gradient) on the device.
int run_mpg(DevInstance & d, const HostVectors & hv, double * x, size_t niter,
            double max_pg, double max_value, FILE * log, size_t period,
            double * diag5, double offset, SolveStats & st);

// Solver scratch carved out of caller-provided device memory (the
// allocation-free entry point, static_solve.cu): control words, reduction
// slots for up to max_blocks CTAs, outputs, step sizes, x in device order
// and the APPROX workspace.
struct ScratchSolve {
        void * ctl = nullptr;
        double * slots = nullptr;
        int max_blocks = 0;
        double * result = nullptr;
        void * out = nullptr;
        int * log_count = nullptr;
        double * v = nullptr, * inv_v = nullptr, * xd = nullptr;
        double * wn[9] = {};
        double * wm[3] = {};  // 2m each, as DevInstance::wm
};
// Bytes of the control region of a ScratchSolve for max_blocks CTAs
// (everything but the vectors).
size_t scratch_control_bytes(int max_blocks);
// Lays out the control region (scratch_control_bytes(max_blocks) bytes at
// base) into s: control words, reduction slots, result, output, log count.
void carve_control(char * base, int max_blocks, ScratchSolve & s);

// approx_solve from a device array x (n doubles, original order, updated in
// place) with every piece of solver scratch in `s`; the instance's device
// copy must exist.  Allocates nothing.  Returns the reason or a negative
// code; diag5 (host, may be NULL) receives the diagnosis.
int run_approx_scratch(DevInstance & d, const HostVectors & hv, double * x_dev,
                       size_t niter, double max_pg, double max_value,
                       double min_delta, double * diag5, double offset,
                       const ScratchSolve & s, cudaStream_t stream);

// Step sizes of the uploaded instance (approx.c:135-186) into host arrays
// in original order: beta (m), v (n), inv_v (n).
int dev_step_sizes(DevInstance & d, const HostVectors & hv, double * beta,
                   double * v, double * inv_v);

}  // namespace acd
