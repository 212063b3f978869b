// The solver kernels: their argument blocks and the __global__ entry
// points.  Each kernel is compiled in one translation unit of its own
// (k_*.cu), which hands its address to the host code in solver.cu through
// the kernel_* functions declared at the end; solver.cu itself compiles no
// solver kernel.  Splitting them lets the build run the slow device
// compilations in parallel.
#pragma once
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <cstring>

#include "device.cuh"
#include "solver.cuh"

namespace acd {

constexpr int kThreads = 512;       // grid-team CTAs (1 per SM)
constexpr int kBatchThreads = 512;  // one-CTA and cluster teams: 16 warps of memory parallelism

struct AlmKernelArgs {
        AlmProblem P;
        AlmMixed M;
        InnerWork<double> W;
        LogBuf log;
        AlmArgs a;
        double * x;
        double * lam;
        TeamCtl * ctl;
        double * slots;
        double * result;
        AlmOut * out;
};

// Trace: the grid team records phase timestamps (a separate instantiation,
// so the untraced solve pays nothing for it).
template <bool Exact, bool Trace = false>
__global__ void __launch_bounds__(kThreads, 1) alm_kernel(AlmKernelArgs k)
{
        GridTeamT<Trace> tm{k.ctl, k.slots, k.result, 0, 0u};
        Alm<GridTeamT<Trace>, Exact> alm(tm, k.P, k.W, k.log, k.M);
        AlmOut out;
        memset(&out, 0, sizeof(out));
        int r = alm.solve(k.a, k.x, k.lam, out);
        if (blockIdx.x == 0 && threadIdx.x == 0) {
                if (r < 0)
                        out.ret = r;
                *k.out = out;
        }
}

struct ApproxOut {
        int reason;
        double diag[5];
        long long iters;
};

struct ApproxKernelArgs {
        InnerProblem<double> P;
        InnerWork<double> W;
        LogBuf log;
        InnerArgs a;
        double * x;
        TeamCtl * ctl;
        double * slots;
        double * result;
        ApproxOut * out;
};

template <bool Exact>
__global__ void __launch_bounds__(kThreads, 1) approx_kernel(ApproxKernelArgs k)
{
        GridTeam tm{k.ctl, k.slots, k.result, 0, 0u};
        Approx<double, GridTeam, Exact> ap(tm, k.P, k.W, k.log);
        ApproxOut out;
        memset(&out, 0, sizeof(out));
        InnerArgs a = k.a;
        a.t_start_ns = global_ns();
        out.reason = ap.solve(a, k.x, out.diag, &out.iters);
        if (blockIdx.x == 0 && threadIdx.x == 0)
                *k.out = out;
}

// ---- spectral projected gradient (mpg_solve / spg_iter) ------------------
//
// approx.c:517-573 and mpg.inc:155-199.  The projection at the top of
// spg_iter is skipped: x is always the output of a projection already
// (the initial projection or the previous step), and clamping is
// idempotent.
template <class Team, bool Exact>
struct Spg {
        Approx<double, Team, Exact> & ap;
        __device__ Spg(Approx<double, Team, Exact> & a) : ap(a) {}

        __device__ int solve(const InnerArgs & a, double * x_io, double * diag,
                             long long * iters_out)
        {
                auto & tm = ap.tm;
                auto & P = ap.P;
                auto & W = ap.W;
                // state (approx.c:531-539): x = P(x0), z = x, g = grad(x), g2 = g
                Vec<double> x = {W.xx, W.vx, 0, NAN, NAN};
                double * z = W.zx;
                double * g = W.g;
                double * g2 = W.g2;
                for (int j = tm.tid(); j < P.n; j += tm.nthreads()) {
                        double xj = tm.ld(x_io + j);
                        double lo = maxpd(tm.ld(P.l + j), xj);
                        double v = minpd(lo, tm.ld(P.u + j));
                        x.x[j] = v;
                        z[j] = v;
                }
                if (!tm.sync())
                        return -1;
                double cx;
                ap.x = x;
                if (!ap.violation(ap.x, 0, 0, 0, true, false, &cx, nullptr, nullptr))
                        return -1;
                x = ap.x;
                {
                        double pg2, gg;
                        if (!ap.gradient(x, false, pg2, gg))
                                return -1;
                }
                for (int j = tm.tid(); j < P.n; j += tm.nthreads())
                        g2[j] = tm.ld(g + j);
                if (!tm.sync())
                        return -1;
                int reason = 0;
                long long i;
                for (i = 0; i < a.niter && !reason; i++) {
                        // gradient at x, pg, y = x - z, u = g - g2, dots
                        double part[4] = {0, 0, 0, 0};
                        const int op[4] = {RED_SUM, RED_SUM, RED_SUM, RED_SUM};
                        {
                                sell_rows_1<Exact, kViolStride>(tm, P.At, x.viol, [&](int j, double s) {
                                        double gj = s + tm.ld(P.c + j);
                                        g[j] = gj;
                                        double xj = tm.ld(x.x + j);
                                        double xp = xj - gj;
                                        xp = maxpd(tm.ld(P.l + j), xp);
                                        xp = minpd(tm.ld(P.u + j), xp);
                                        double d = xj - xp;
                                        part[0] += d * d;
                                        double yj = xj - tm.ld(z + j);
                                        double uj = gj - tm.ld(g2 + j);
                                        part[1] += yj * yj;
                                        part[2] += yj * uj;
                                });
                        }
                        if (!tm.reduce(part, op))
                                return -1;
                        double pg = sqrt(part[0]);
                        double stepl = part[1] / part[2];
                        if (stepl != stepl)
                                stepl = 1;
                        if (!(stepl > 1e8)) {
                                // z = P(x - step g); swap(z, x); swap(g2, g)
                                for (int j = tm.tid(); j < P.n; j += tm.nthreads()) {
                                        double v = tm.ld(x.x + j) - stepl * tm.ld(g + j);
                                        v = maxpd(tm.ld(P.l + j), v);
                                        v = minpd(tm.ld(P.u + j), v);
                                        z[j] = v;
                                }
                                if (!tm.sync())
                                        return -1;
                                double * t = z;
                                z = x.x;
                                x.x = t;
                                t = g2;
                                g2 = g;
                                g = t;
                                ap.W.g = g;
                        }
                        // value of the new x (its violation feeds the next
                        // gradient)
                        ap.x = x;
                        if (!ap.violation(ap.x, 0, 0, 0, true, false, &cx, nullptr, nullptr))
                                return -1;
                        x = ap.x;
                        double value = a.offset + x.quad + cx;
                        if (pg < a.max_pg)
                                reason = 2;
                        if (value < a.max_value)
                                reason = 1;
                        if (a.log && ((a.period && (i % a.period == 0)) || i == 0 || reason)) {
                                LogRec r = {2, 0, 0, 0, i + 1, {pg, value, 0, 0, 0, 0}};
                                ap.put_log(r);
                        }
                }
                // diagnosis (approx.c:556-569)
                double pg2, gg;
                if (!ap.gradient(x, false, pg2, gg))
                        return -1;
                for (int j = tm.tid(); j < P.n; j += tm.nthreads())
                        x_io[j] = tm.ld(x.x + j);
                if (!tm.sync())
                        return -1;
                diag[0] = a.offset + x.quad + cx;
                diag[1] = sqrt(gg);
                diag[2] = sqrt(pg2);
                diag[3] = HUGE_VAL;
                diag[4] = (double)(i + 1);
                *iters_out = i;
                (void)reason;
                return 2;
        }
};

template <bool Exact>
__global__ void __launch_bounds__(kThreads, 1) mpg_kernel(ApproxKernelArgs k)
{
        GridTeam tm{k.ctl, k.slots, k.result, 0, 0u};
        Approx<double, GridTeam, Exact> ap(tm, k.P, k.W, k.log);
        Spg<GridTeam, Exact> spg(ap);
        ApproxOut out;
        memset(&out, 0, sizeof(out));
        out.reason = spg.solve(k.a, k.x, out.diag, &out.iters);
        if (blockIdx.x == 0 && threadIdx.x == 0)
                *k.out = out;
}

// ---- one LP per CTA (batches, small served LPs) ----


// One LP on one CTA, its arguments passed by value (the server's launches).
template <bool Exact>
__global__ void __launch_bounds__(kBatchThreads, 1) alm_single_kernel(AlmKernelArgs k)
{
        BlockTeam tm{reinterpret_cast<int *>(&k.ctl->status_w.v)};
        Alm<BlockTeam, Exact> alm(tm, k.P, k.W, k.log, k.M);
        AlmOut out;
        memset(&out, 0, sizeof(out));
        int r = alm.solve(k.a, k.x, k.lam, out);
        if (threadIdx.x == 0) {
                if (r < 0)
                        out.ret = r;
                *k.out = out;
        }
}

// Persistent CTAs take LPs from a shared counter (largest first) and run
// each one's whole ALM solve with a one-CTA team.
template <bool Exact>
__global__ void __launch_bounds__(kBatchThreads, 1)
alm_batch_kernel(const AlmKernelArgs * items, int count, int * next)
{
        __shared__ int cur;
        for (;;) {
                if (threadIdx.x == 0)
                        cur = atomicAdd(next, 1);
                __syncthreads();
                int i = cur;
                __syncthreads();
                if (i >= count)
                        break;
                const AlmKernelArgs & k = items[i];
                BlockTeam tm{reinterpret_cast<int *>(&k.ctl->status_w.v)};
                Alm<BlockTeam, Exact> alm(tm, k.P, k.W, k.log, k.M);
                AlmOut out;
                memset(&out, 0, sizeof(out));
                int r = alm.solve(k.a, k.x, k.lam, out);
                if (threadIdx.x == 0) {
                        if (r < 0)
                                out.ret = r;
                        *k.out = out;
                }
                __syncthreads();
        }
}

// One LP on one thread-block cluster (launched with a cluster dimension).
template <bool Exact>
__global__ void __launch_bounds__(kBatchThreads, 1) alm_cluster_kernel(AlmKernelArgs k)
{
        ClusterTeam tm(reinterpret_cast<int *>(&k.ctl->status_w.v));
        Alm<ClusterTeam, Exact> alm(tm, k.P, k.W, k.log, k.M);
        AlmOut out;
        memset(&out, 0, sizeof(out));
        int r = alm.solve(k.a, k.x, k.lam, out);
        if (tm.rank == 0 && threadIdx.x == 0) {
                if (r < 0)
                        out.ret = r;
                *k.out = out;
        }
        // no CTA leaves while the others may still read its shared memory
        tm.sync();
}

// Kernel addresses, one translation unit each (k_*.cu).
const void * kernel_alm_grid_fast();      // k_alm_grid.cu
const void * kernel_alm_grid_exact();     // k_alm_grid_exact.cu
const void * kernel_alm_grid_trace();     // k_alm_grid_trace.cu (fused, traced)
const void * kernel_approx_grid(bool exact);  // k_approx_grid.cu
const void * kernel_mpg_grid();               // k_approx_grid.cu
const void * kernel_alm_single_fast();    // k_alm_block.cu
const void * kernel_alm_batch_fast();     // k_alm_block.cu
const void * kernel_alm_single_exact();   // k_alm_block_exact.cu
const void * kernel_alm_batch_exact();    // k_alm_block_exact.cu
const void * kernel_alm_cluster(bool exact);  // k_alm_cluster.cu

inline const void * kernel_alm_grid(bool exact)
{
        return exact ? kernel_alm_grid_exact() : kernel_alm_grid_fast();
}
inline const void * kernel_alm_single(bool exact)
{
        return exact ? kernel_alm_single_exact() : kernel_alm_single_fast();
}
inline const void * kernel_alm_batch(bool exact)
{
        return exact ? kernel_alm_batch_exact() : kernel_alm_batch_fast();
}

}  // namespace acd
