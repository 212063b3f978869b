// Host launchers of the solver kernels (kernels.cuh) and the small kernels
// they need (permutation, step sizes).
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.h"
#include "device.cuh"
#include "instance.h"
#include "kernels.cuh"
#include "solver.cuh"

namespace acd {

namespace {

constexpr int kMaxTeamCtas = 1024;  // GridTeam's per-lane wait mask covers 32 x 32 CTAs
constexpr int kLogCap = 1 << 14;

// ---- small kernels ------------------------------------------------------

// dst[d] = src[map[d]]: original order -> device order
__global__ void gather_kernel(double * dst, const double * src,
                              const int32_t * map, int n)
{
        for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n;
             d += gridDim.x * blockDim.x)
                dst[d] = src[map[d]];
}

// dst[map[d]] = src[d]: device order -> original order
__global__ void scatter_kernel(double * dst, const double * src,
                               const int32_t * map, int n)
{
        for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < n;
             d += gridDim.x * blockDim.x)
                dst[map[d]] = src[d];
}

// approx_update_step_size (approx.c:135-186) in device order: the A' rows
// list each column's entries in the reference's summation order and the
// arithmetic rounds like the reference, so v is bit-identical.
__global__ void step_size_kernel(SellDev<double> at, const double * w,
                                 const double * beta, const double * c,
                                 double * v, double * inv_v)
{
        int lane = threadIdx.x & 31;
        int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        int nwarps = (gridDim.x * blockDim.x) >> 5;
        for (int s = warp; s < at.nslices; s += nwarps) {
                Slice sl = slice_of(at, s, lane);
                double acc = by_width(sl, [&](auto wv) {
                        constexpr int VEC = decltype(wv)::value;
                        int64_t e = sl.base + VEC * lane;
                        double sum = 0;
                        for (int k = 0; k < sl.steps; k++, e += 32 * VEC) {
                                Chunk<VEC, double> q = load_chunk<VEC>(at.col, at.val, e);
                                double t[VEC];
#pragma unroll
                                for (int j = 0; j < VEC; j++)
                                        t[j] = __dmul_rn(__dmul_rn(__dmul_rn(w[q.c[j]], beta[q.c[j]]),
                                                                   q.a[j]),
                                                         q.a[j]);
                                sum = in_order<VEC>(sum, t, sl.shift, lane);
                        }
                        return sum;
                });
                int j = sl.row;
                if (sl.lead && j < at.nrows) {
                        v[j] = acc;
                        inv_v[j] = (acc == 0 && c[j] == 0) ? 1.0 : 1.0 / acc;
                }
        }
}


// ---- host helpers --------------------------------------------------------

}  // namespace

// Reference rounding in the solver kernels (separate rounding of products
// and sums, as the reference's C code) instead of fused multiply-adds.
bool g_exact = getenv("ACDALM_EXACT") && getenv("ACDALM_EXACT")[0] == '1';

namespace {

template <class T>
T * carve(char *& p, size_t count)
{
        T * r = reinterpret_cast<T *>(p);
        size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
        p += bytes;
        return r;
}

size_t rounded(size_t bytes)
{
        return (bytes + 255) & ~size_t(255);
}

int launch_blocks(const void * kernel)
{
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kThreads, 0);
        if (per_sm < 1)
                per_sm = 1;
        return sms * per_sm;
}

void print_logs(FILE * log, const std::vector<LogRec> & recs)
{
        if (log == nullptr)
                return;
        for (const LogRec & r : recs) {
                if (r.kind == 0) {
                        // approx.c:617-627 restart markers, approx.c:504-515
                        if (r.restarts > 0) {
                                fprintf(log, "\t\t ");
                                for (int i = 0; i < r.restarts; i++)
                                        fputc('R', log);
                        }
                        if (r.has_delta)
                                fprintf(log, "\t%10lld %12g %12g %12g %8g %12g\n", r.k,
                                        r.a[0], r.a[1], r.a[2], r.a[3], r.a[4]);
                        else
                                fprintf(log, "\t%10lld %12g %12g %12g %8g\n", r.k,
                                        r.a[0], r.a[1], r.a[2], r.a[3]);
                } else if (r.kind == 1) {
                        // alm.c:260-285
                        fprintf(log, "%4lld: %12g %12g %12g %.18g %.18g", r.k, r.a[0],
                                r.a[1], r.a[2], r.a[3], r.a[4]);
                        if (r.stalled)
                                fprintf(log, " -stalled-\n");
                        else
                                fprintf(log, " (%8g)\n", r.a[5]);
                } else {
                        // approx.c:550-553
                        fprintf(log, "%10lld: %12g %12g\n", r.k, r.a[0], r.a[1]);
                }
        }
        fflush(log);
}

int fetch_logs(DevInstance & d, FILE * log)
{
        if (log == nullptr)
                return 0;
        int count = 0;
        ACD_CUDA_TRY(cudaMemcpyAsync(&count, d.log_count, sizeof(int),
                                     cudaMemcpyDeviceToHost, d.stream), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaStreamSynchronize(d.stream), ACDALM_ECUDA);
        int n = std::min(count, d.log_cap);
        std::vector<LogRec> recs(n);
        if (n > 0)
                ACD_CUDA_TRY(cudaMemcpy(recs.data(), d.log, n * sizeof(LogRec),
                                        cudaMemcpyDeviceToHost), ACDALM_ECUDA);
        print_logs(log, recs);
        if (count > d.log_cap)
                fprintf(log, "(%d log lines dropped)\n", count - d.log_cap);
        return 0;
}

// Upload an original-order host vector into a device-order array.
int upload_gather(DevInstance & d, double * dst, const double * src,
                  const int32_t * map, int len, double fill)
{
        if (len == 0)
                return 0;
        std::vector<double> tmp;
        if (src == nullptr) {
                tmp.assign(len, fill);
                src = tmp.data();
        }
        // staged through the instance's spare buffer of that length
        double * tmpdev = (len <= d.n) ? d.wn[8] : d.wm[2];
        ACD_CUDA_TRY(cudaMemcpyAsync(tmpdev, src, len * sizeof(double),
                                     cudaMemcpyHostToDevice, d.stream), ACDALM_ECUDA);
        gather_kernel<<<std::min(1024, (len + 255) / 256), 256, 0, d.stream>>>(
                dst, tmpdev, map, len);
        count_launch();
        ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        if (!tmp.empty())
                ACD_CUDA_TRY(cudaStreamSynchronize(d.stream), ACDALM_ECUDA);
        return 0;
}

int download_scatter(DevInstance & d, double * dst, const double * src,
                     const int32_t * map, int len)
{
        if (len == 0)
                return 0;
        double * tmpdev = (len <= d.n) ? d.wn[8] : d.wm[2];
        scatter_kernel<<<std::min(1024, (len + 255) / 256), 256, 0, d.stream>>>(
                tmpdev, src, map, len);
        count_launch();
        ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaMemcpyAsync(dst, tmpdev, len * sizeof(double),
                                     cudaMemcpyDeviceToHost, d.stream), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaStreamSynchronize(d.stream), ACDALM_ECUDA);
        return 0;
}

int upload_problem(DevInstance & d, const HostVectors & hv)
{
        int r;
        if ((r = upload_gather(d, d.b, hv.b, d.row_orig, d.m, 0)) ||
            (r = upload_gather(d, d.w, hv.w, d.row_orig, d.m, 1)) ||
            (r = upload_gather(d, d.c0, hv.c0, d.col_orig, d.n, 0)) ||
            (r = upload_gather(d, d.l, hv.l, d.col_orig, d.n, -HUGE_VAL)) ||
            (r = upload_gather(d, d.u, hv.u, d.col_orig, d.n, HUGE_VAL)))
                return r;
        // multiplier bounds: ALM only
        if (hv.lam_lo || hv.lam_hi)
                if ((r = upload_gather(d, d.lam_lo, hv.lam_lo, d.row_orig, d.m, -HUGE_VAL)) ||
                    (r = upload_gather(d, d.lam_hi, hv.lam_hi, d.row_orig, d.m, HUGE_VAL)))
                        return r;
        ACD_CUDA_TRY(cudaStreamSynchronize(d.stream), ACDALM_ECUDA);
        return 0;
}

InnerWork<double> work_of(DevInstance & d)
{
        InnerWork<double> W;
        W.zx = d.wn[0];
        W.zpx = d.wn[1];
        W.xx = d.wn[2];
        W.g = d.wn[3];
        W.g2 = d.wn[4];
        W.prev = d.wn[5];
        W.prev_alt = d.wn[6];
        W.alt_x = d.wn[7];
        W.ux = d.wn[8];
        W.vz = d.wm[0];
        W.vzp = d.wm[1];
        W.vx = d.wm[2];
        return W;
}

SellDev<double> sell_a(const DevInstance & d)
{
        return {d.m, d.a_nslices, d.a_ptr, d.a_row0, d.a_col, d.a_val};
}

SellDev<double> sell_at(const DevInstance & d)
{
        return {d.n, d.at_nslices, d.at_ptr, d.at_row0, d.at_col, d.at_val};
}

int reset_ctl(DevInstance & d)
{
        ACD_CUDA_TRY(cudaMemsetAsync(d.ctl, 0, sizeof(TeamCtl), d.stream), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaMemsetAsync(d.log_count, 0, sizeof(int), d.stream), ACDALM_ECUDA);
        return 0;
}

int read_status(DevInstance & d, int & status)
{
        int s = 0;
        ACD_CUDA_TRY(cudaMemcpy(&s, &static_cast<TeamCtl *>(d.ctl)->status_w.v, sizeof(int),
                                cudaMemcpyDeviceToHost), ACDALM_ECUDA);
        status = s;
        return 0;
}

const char * status_text(int status)
{
        switch (status) {
        case ACDALM_ETIMEOUT:
                return "a device wait for the other CTAs of the team ran out";
        case ACDALM_ETIMELIMIT:
                return "the solve ran past its time limit, ACDALM_SOLVE_TIMEOUT";
        case ACDALM_ENONFINITE:
                return "an iterate stopped being finite";
        default:
                return "device failure";
        }
}

// Whole-solve time limit on the device (ACDALM_SOLVE_TIMEOUT seconds,
// default 900): a solve that runs longer stops with ACDALM_ETIMELIMIT.
unsigned long long solve_limit_ns()
{
        const char * e = getenv("ACDALM_SOLVE_TIMEOUT");
        double sec = e ? atof(e) : 900.0;
        if (!(sec > 0))
                return 0;
        return (unsigned long long)(sec * 1e9);
}

int launch_coop(const void * fn, int max_blocks, void * args, double * slots,
                cudaStream_t s, int * launched = nullptr)
{
        // every CTA must be resident at once: never more than the occupancy
        // of this kernel allows, nor more than the reduction slots hold
        int blocks = std::min(std::min(max_blocks, launch_blocks(fn)), kMaxTeamCtas);
        // The grid team's reduction lines carry the epoch that wrote them,
        // counted from 1 in every launch: a line left by an earlier launch
        // on the same slots (one that ended after a few reductions, or
        // failed) could carry a tag this launch waits for.  Zeroed lines
        // never match.
        ACD_CUDA_TRY(cudaMemsetAsync(slots, 0, 2 * (size_t)blocks * kSlotStride * sizeof(double),
                                     s), ACDALM_ECUDA);
        void * params[1] = {args};
        ACD_CUDA_TRY(cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(kThreads),
                                                 params, 0, s), ACDALM_ECUDA);
        count_launch();
        if (launched)
                *launched = blocks;
        return 0;
}

}  // namespace

// ---- DevInstance ---------------------------------------------------------

int DevInstance::create(const DeviceLayout & lay)
{
        m = lay.m;
        n = lay.n;
        nnz = lay.nnz;
        a_nslices = lay.a.nslices;
        at_nslices = lay.at.nslices;
        max_width_a = lay.a.max_width;
        max_width_at = lay.at.max_width;
        int blocks = std::max(std::max(launch_blocks(kernel_alm_grid(false)),
                                       launch_blocks(kernel_approx_grid(false))),
                              std::max(launch_blocks(kernel_alm_grid(true)),
                                       launch_blocks(kernel_mpg_grid())));
        grid_blocks = blocks;
        size_t ea = lay.a.ptr.back(), eat = lay.at.ptr.back();
        size_t sa = std::max<size_t>(lay.a.row0.size(), 1), sat = std::max<size_t>(lay.at.row0.size(), 1);
        size_t mm = std::max(m, 1), nn = std::max(n, 1);
        size_t total = 0;
        total += rounded((lay.a.ptr.size()) * 8) + rounded(sa * 4) + rounded(ea * 4) + rounded(ea * 8);
        total += rounded((lay.at.ptr.size()) * 8) + rounded(sat * 4) + rounded(eat * 4) + rounded(eat * 8);
        total += rounded(mm * 4) + rounded(nn * 4) + rounded(mm * 8);
        total += 6 * rounded(mm * 8) + 7 * rounded(nn * 8);
        total += 9 * rounded(nn * 8) + 3 * rounded(mm * 16);
        total += rounded(sizeof(TeamCtl)) + rounded(2 * (size_t)blocks * kSlotStride * 8)
                + rounded(2 * kRedMax * 8);
        log_cap = kLogCap;
        total += rounded((size_t)log_cap * sizeof(LogRec)) + rounded(sizeof(int));
        total += rounded(std::max(sizeof(AlmOut), sizeof(ApproxOut)));
        ACD_CUDA_TRY(cudaStreamCreateWithPriority(&stream, cudaStreamNonBlocking, priority),
                     ACDALM_ECUDA);
        // stream-ordered allocation: no device-wide synchronisation, so a
        // server can admit and retire instances while others run
        cudaError_t e = cudaMallocAsync(&mem, total, stream);
        if (e != cudaSuccess) {
                set_error(ACDALM_ENOMEM, "cudaMalloc(%zu bytes): %s", total,
                          cudaGetErrorString(e));
                mem = nullptr;
                return ACDALM_ENOMEM;
        }
        bytes = total;
        char * p = static_cast<char *>(mem);
        a_ptr = carve<int64_t>(p, lay.a.ptr.size());
        a_row0 = carve<int32_t>(p, sa);
        a_col = carve<int32_t>(p, ea);
        a_val = carve<double>(p, ea);
        at_ptr = carve<int64_t>(p, lay.at.ptr.size());
        at_row0 = carve<int32_t>(p, sat);
        at_col = carve<int32_t>(p, eat);
        at_val = carve<double>(p, eat);
        row_orig = carve<int32_t>(p, mm);
        col_orig = carve<int32_t>(p, nn);
        beta = carve<double>(p, mm);
        b = carve<double>(p, mm);
        w = carve<double>(p, mm);
        lam_lo = carve<double>(p, mm);
        lam_hi = carve<double>(p, mm);
        lam = carve<double>(p, mm);
        r = carve<double>(p, mm);
        c0 = carve<double>(p, nn);
        l = carve<double>(p, nn);
        u = carve<double>(p, nn);
        c = carve<double>(p, nn);
        v = carve<double>(p, nn);
        inv_v = carve<double>(p, nn);
        x = carve<double>(p, nn);
        for (auto & q : wn)
                q = carve<double>(p, nn);
        for (auto & q : wm)
                q = carve<double>(p, 2 * mm);
        ctl = carve<TeamCtl>(p, 1);
        slots = carve<double>(p, 2 * (size_t)blocks * kSlotStride);
        result = carve<double>(p, 2 * kRedMax);
        log = carve<LogRec>(p, log_cap);
        log_count = carve<int>(p, 1);
        out = carve<char>(p, std::max(sizeof(AlmOut), sizeof(ApproxOut)));

        ACD_CUDA_TRY(cudaMemsetAsync(mem, 0, total, stream), ACDALM_ECUDA);
        auto up = [&](void * dst, const void * src, size_t nb) {
                return nb ? cudaMemcpyAsync(dst, src, nb, cudaMemcpyHostToDevice, stream)
                          : cudaSuccess;
        };
        ACD_CUDA_TRY(up(a_ptr, lay.a.ptr.data(), lay.a.ptr.size() * 8), ACDALM_ECUDA);
        ACD_CUDA_TRY(up(a_row0, lay.a.row0.data(), lay.a.row0.size() * 4), ACDALM_ECUDA);
        ACD_CUDA_TRY(up(a_col, lay.a.col.data(), ea * 4), ACDALM_ECUDA);
        ACD_CUDA_TRY(up(a_val, lay.a.val.data(), ea * 8), ACDALM_ECUDA);
        ACD_CUDA_TRY(up(at_ptr, lay.at.ptr.data(), lay.at.ptr.size() * 8), ACDALM_ECUDA);
        ACD_CUDA_TRY(up(at_row0, lay.at.row0.data(), lay.at.row0.size() * 4), ACDALM_ECUDA);
        ACD_CUDA_TRY(up(at_col, lay.at.col.data(), eat * 4), ACDALM_ECUDA);
        ACD_CUDA_TRY(up(at_val, lay.at.val.data(), eat * 8), ACDALM_ECUDA);
        ACD_CUDA_TRY(up(row_orig, lay.row_orig_of_d.data(), (size_t)m * 4), ACDALM_ECUDA);
        ACD_CUDA_TRY(up(col_orig, lay.col_orig_of_d.data(), (size_t)n * 4), ACDALM_ECUDA);
        ACD_CUDA_TRY(up(beta, lay.beta.data(), (size_t)m * 8), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaStreamSynchronize(stream), ACDALM_ECUDA);
        return 0;
}

size_t DevInstance::footprint(const DeviceLayout & lay, bool mixed)
{
        size_t ea = lay.a.ptr.back(), eat = lay.at.ptr.back();
        size_t sa = std::max<size_t>(lay.a.row0.size(), 1), sat = std::max<size_t>(lay.at.row0.size(), 1);
        size_t mm = std::max(lay.m, 1), nn = std::max(lay.n, 1);
        size_t total = rounded((lay.a.ptr.size()) * 8) + rounded(sa * 4) + rounded(ea * 4) + rounded(ea * 8);
        total += rounded((lay.at.ptr.size()) * 8) + rounded(sat * 4) + rounded(eat * 4) + rounded(eat * 8);
        total += rounded(mm * 4) + rounded(nn * 4) + rounded(mm * 8);
        total += 6 * rounded(mm * 8) + 7 * rounded(nn * 8);
        total += 9 * rounded(nn * 8) + 3 * rounded(mm * 16);
        total += (size_t)2 << 20;  // control, slots, log ring, outputs (bounded)
        if (mixed)
                total += rounded(ea * 4) + rounded(eat * 4) + 2 * rounded(mm * 4) + 15 * rounded(nn * 4)
                        + 3 * rounded(mm * 8);
        return total;
}

int DevInstance::ensure_f32(const DeviceLayout & lay)
{
        if (mem32)
                return 0;
        size_t ea = lay.a.val.size(), eat = lay.at.val.size();
        size_t mm = std::max(m, 1), nn = std::max(n, 1);
        size_t total = rounded(std::max<size_t>(ea, 1) * 4) + rounded(std::max<size_t>(eat, 1) * 4)
                + 2 * rounded(mm * 4) + 6 * rounded(nn * 4) + 9 * rounded(nn * 4)
                + 3 * rounded(mm * 8);
        cudaError_t e = cudaMallocAsync(&mem32, total, stream);
        if (e != cudaSuccess) {
                mem32 = nullptr;
                set_error(ACDALM_ENOMEM, "cudaMalloc(%zu bytes) for the FP32 copies: %s",
                          total, cudaGetErrorString(e));
                return ACDALM_ENOMEM;
        }
        bytes32 = total;
        char * p = static_cast<char *>(mem32);
        a_valf = carve<float>(p, std::max<size_t>(ea, 1));
        at_valf = carve<float>(p, std::max<size_t>(eat, 1));
        bf = carve<float>(p, mm);
        wf = carve<float>(p, mm);
        cf = carve<float>(p, nn);
        lf = carve<float>(p, nn);
        uf = carve<float>(p, nn);
        vf = carve<float>(p, nn);
        ivf = carve<float>(p, nn);
        d = carve<float>(p, nn);
        for (auto & q : wnf)
                q = carve<float>(p, nn);
        for (auto & q : wmf)
                q = carve<float>(p, 2 * mm);
        ACD_CUDA_TRY(cudaMemsetAsync(mem32, 0, total, stream), ACDALM_ECUDA);
        std::vector<float> tmp(lay.a.val.begin(), lay.a.val.end());
        if (ea)
                ACD_CUDA_TRY(cudaMemcpyAsync(a_valf, tmp.data(), ea * 4, cudaMemcpyHostToDevice,
                                             stream), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaStreamSynchronize(stream), ACDALM_ECUDA);
        tmp.assign(lay.at.val.begin(), lay.at.val.end());
        if (eat)
                ACD_CUDA_TRY(cudaMemcpyAsync(at_valf, tmp.data(), eat * 4, cudaMemcpyHostToDevice,
                                             stream), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaStreamSynchronize(stream), ACDALM_ECUDA);
        return 0;
}

void DevInstance::destroy()
{
        if (trace_rec)
                cudaFreeAsync(trace_rec, stream);
        trace_rec = nullptr;
        trace_cap = trace_ctas = trace_count = 0;
        if (mem32)
                cudaFreeAsync(mem32, stream);
        mem32 = nullptr;
        if (mem)
                cudaFreeAsync(mem, stream);
        mem = nullptr;
        if (stream)
                cudaStreamDestroy(stream);
        stream = nullptr;
}

// ---- entry points --------------------------------------------------------

int dev_step_sizes(DevInstance & d, const HostVectors & hv, double * beta_out,
                   double * v_out, double * inv_v_out)
{
        int r = upload_problem(d, hv);
        if (r)
                return r;
        step_size_kernel<<<std::max(1, std::min(4096, (d.n + 255) / 256)), 256, 0,
                           d.stream>>>(sell_at(d), d.w, d.beta, d.c0, d.v, d.inv_v);
        count_launch();
        ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        if (v_out && (r = download_scatter(d, v_out, d.v, d.col_orig, d.n)))
                return r;
        if (inv_v_out && (r = download_scatter(d, inv_v_out, d.inv_v, d.col_orig, d.n)))
                return r;
        if (beta_out && (r = download_scatter(d, beta_out, d.beta, d.row_orig, d.m)))
                return r;
        return 0;
}

static double env_or(const char * name, double dflt)
{
        const char * e = getenv(name);
        return e ? atof(e) : dflt;
}

// Uploads one instance's problem, x and lambda and fills the kernel
// arguments of its ALM solve.
static int alm_prepare(DevInstance & d, const HostVectors & hv, size_t niter, double * x,
                       double * lam, bool want_log, const AlmSettings & s,
                       const DeviceLayout * lay, AlmKernelArgs & k)
{
        bool mixed = mixed_for(s.precision, d.nnz);
        if (mixed) {
                if (!lay) {
                        set_error(ACDALM_EINVAL, "mixed precision needs the device layout");
                        return ACDALM_EINVAL;
                }
                int e = d.ensure_f32(*lay);
                if (e)
                        return e;
        }
        int r = upload_problem(d, hv);
        if (r)
                return r;
        if ((r = upload_gather(d, d.x, x, d.col_orig, d.n, 0)) ||
            (r = upload_gather(d, d.lam, lam, d.row_orig, d.m, 0)) || (r = reset_ctl(d)))
                return r;
        // |b|, |c0| for the relative KKT terms
        double bn = 0, cn = 0;
        for (int i = 0; i < d.m; i++)
                bn += hv.b[i] * hv.b[i];
        if (hv.c0)
                for (int j = 0; j < d.n; j++)
                        cn += hv.c0[j] * hv.c0[j];
        memset(&k, 0, sizeof(k));
        k.P.m = d.m;
        k.P.n = d.n;
        k.P.A = sell_a(d);
        k.P.At = sell_at(d);
        k.P.b = d.b;
        k.P.c0 = d.c0;
        k.P.l = d.l;
        k.P.u = d.u;
        k.P.lam_lo = d.lam_lo;
        k.P.lam_hi = d.lam_hi;
        k.P.beta = d.beta;
        k.P.orig_row = d.row_orig;
        k.P.w = d.w;
        k.P.c = d.c;
        k.P.v = d.v;
        k.P.inv_v = d.inv_v;
        k.P.r = d.r;
        k.P.bnorm = sqrt(bn);
        k.P.cnorm = sqrt(cn);
        k.W = work_of(d);
        k.log = {d.log, d.log_cap, d.log_count};
        k.a.niter = (long long)std::min<size_t>(niter, (size_t)1 << 62);
        k.a.inner_budget = s.inner_budget;
        k.a.kkt_tol = s.kkt_tol;
        k.a.log = want_log;
        k.a.limit_ns = solve_limit_ns();
        k.a.mixed = mixed ? 1 : 0;
        k.a.min_delta32 = env_or("ACDALM_MIN_DELTA32", 1e-6);
        k.a.niter32 = (long long)env_or("ACDALM_NITER32", 200000);
        k.a.stall_switch = (int)env_or("ACDALM_STALL_SWITCH", 2);
        k.a.pg_floor32 = env_or("ACDALM_PG_FLOOR32", 1e-6);
        if (mixed) {
                k.M.Af = {d.m, d.a_nslices, d.a_ptr, d.a_row0, d.a_col, d.a_valf};
                k.M.Atf = {d.n, d.at_nslices, d.at_ptr, d.at_row0, d.at_col, d.at_valf};
                k.M.bf = d.bf;
                k.M.wf = d.wf;
                k.M.cf = d.cf;
                k.M.lf = d.lf;
                k.M.uf = d.uf;
                k.M.vf = d.vf;
                k.M.ivf = d.ivf;
                k.M.d = d.d;
                InnerWork<float> Wf;
                Wf.zx = d.wnf[0];
                Wf.zpx = d.wnf[1];
                Wf.xx = d.wnf[2];
                Wf.g = d.wnf[3];
                Wf.g2 = d.wnf[4];
                Wf.prev = d.wnf[5];
                Wf.prev_alt = d.wnf[6];
                Wf.alt_x = d.wnf[7];
                Wf.ux = d.wnf[8];
                Wf.vz = d.wmf[0];
                Wf.vzp = d.wmf[1];
                Wf.vx = d.wmf[2];
                k.M.Wf = Wf;
        }
        k.x = d.x;
        k.lam = d.lam;
        k.ctl = static_cast<TeamCtl *>(d.ctl);
        k.slots = d.slots;
        k.result = d.result;
        k.out = static_cast<AlmOut *>(d.out);
        return 0;
}

// The trace buffer of a grid solve when the settings ask for one: grown on
// the instance's stream as needed and zeroed; trace.rec stays null otherwise.
static int prepare_trace(DevInstance & d, const AlmSettings & s, TraceBuf & trace)
{
        trace = {nullptr, 0, 0};
        if (s.trace_count == 0)
                return 0;
        size_t need = (size_t)s.trace_count * d.grid_blocks * kTracePhases;
        if (d.trace_cap < need) {
                if (d.trace_rec)
                        cudaFreeAsync(d.trace_rec, d.stream);
                d.trace_rec = nullptr;
                d.trace_cap = 0;
                void * p = nullptr;
                cudaError_t e = cudaMallocAsync(&p, need * sizeof(unsigned long long), d.stream);
                if (e != cudaSuccess) {
                        set_error(ACDALM_ENOMEM, "trace buffer (%zu bytes): %s",
                                  need * sizeof(unsigned long long), cudaGetErrorString(e));
                        return ACDALM_ENOMEM;
                }
                d.trace_rec = static_cast<unsigned long long *>(p);
                d.trace_cap = need;
        }
        ACD_CUDA_TRY(cudaMemsetAsync(d.trace_rec, 0, need * sizeof(unsigned long long), d.stream),
                     ACDALM_ECUDA);
        trace = {d.trace_rec, s.trace_first, s.trace_count};
        return 0;
}

// Copies the last traced launch's records (see TraceBuf).
int copy_trace(DevInstance & d, unsigned long long * out, size_t cap, size_t * ctas,
               size_t * count)
{
        if (ctas)
                *ctas = d.trace_ctas;
        if (count)
                *count = d.trace_count;
        size_t n = d.trace_ctas * d.trace_count * kTracePhases;
        if (!out || n == 0)
                return 0;
        if (cap < n) {
                set_error(ACDALM_EINVAL, "alm_trace_copy: %zu records need %zu values, buffer "
                          "holds %zu", d.trace_count, n, cap);
                return ACDALM_EINVAL;
        }
        ACD_CUDA_TRY(cudaMemcpy(out, d.trace_rec, n * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost), ACDALM_ECUDA);
        return 0;
}

// Reads one instance's outcome after its ALM kernel finished.
static int alm_finish(DevInstance & d, const AlmKernelArgs & k, double * x, double * lam,
                      FILE * log, double * diag3, double * w_out, double * c_out,
                      SolveStats & st, double seconds)
{
        int status = 0, r;
        if ((r = read_status(d, status)))
                return r;
        AlmOut out;
        ACD_CUDA_TRY(cudaMemcpy(&out, d.out, sizeof(out), cudaMemcpyDeviceToHost), ACDALM_ECUDA);
        fetch_logs(d, log);
        st.seconds = seconds;
        st.inner = out.inner;
        st.outer = (unsigned long long)out.outer;
        st.rel_kkt = out.rel_kkt;
        st.primal = out.primal;
        st.dual = out.dual;
        st.gap = out.gap;
        st.objective = out.objective;
        st.status = status;
        st.precision = k.a.mixed;
        st.inner_fp32 = out.inner32;
        if (status != 0) {
                set_error(status, "device solve failed with status %d (%s)", status,
                          status_text(status));
                return status;
        }
        if ((r = download_scatter(d, x, d.x, d.col_orig, d.n)) ||
            (r = download_scatter(d, lam, d.lam, d.row_orig, d.m)))
                return r;
        if (w_out && (r = download_scatter(d, w_out, d.w, d.row_orig, d.m)))
                return r;
        if (c_out && (r = download_scatter(d, c_out, d.c, d.col_orig, d.n)))
                return r;
        if (diag3) {
                diag3[0] = out.diag[0];
                diag3[1] = out.diag[1];
                diag3[2] = out.diag[2];
        }
        return out.ret;
}

int run_alm(DevInstance & d, const HostVectors & hv, size_t niter, double * x,
            double * lam, FILE * log, double * diag3, const AlmSettings & s,
            double * w_out, double * c_out, SolveStats & st, const DeviceLayout * lay)
{
        NvtxRange solve_range("acdalm alm_solve");
        AlmKernelArgs k;
        int r;
        bool traced = false;
        unsigned trace_count = 0;
        {
                NvtxRange up("acdalm upload");
                if ((r = alm_prepare(d, hv, niter, x, lam, log != nullptr, s, lay, k)))
                        return r;
                TraceBuf trace;
                if ((r = prepare_trace(d, s, trace)))
                        return r;
                // after reset_ctl zeroed the control block (tracing off)
                if (trace.rec)
                        ACD_CUDA_TRY(cudaMemcpyAsync(&static_cast<TeamCtl *>(d.ctl)->trace, &trace,
                                                     sizeof(trace), cudaMemcpyHostToDevice,
                                                     d.stream), ACDALM_ECUDA);
                traced = trace.rec != nullptr;
                trace_count = trace.count;
        }
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float ms = 0;
        {
                NvtxRange kr("acdalm solve kernel");
                cudaEventRecord(e0, d.stream);
                // the traced instantiation runs the fused form
                const void * fn = traced ? kernel_alm_grid_trace() : kernel_alm_grid(g_exact);
                int launched = 0;
                if ((r = launch_coop(fn, d.grid_blocks, &k, d.slots, d.stream, &launched)))
                        return r;
                cudaEventRecord(e1, d.stream);
                ACD_CUDA_TRY(cudaStreamSynchronize(d.stream), ACDALM_ECUDA);
                if (traced) {
                        d.trace_ctas = (size_t)launched;
                        d.trace_count = trace_count;
                }
        }
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        NvtxRange down("acdalm download");
        return alm_finish(d, k, x, lam, log, diag3, w_out, c_out, st, ms * 1e-3);
}

// ---- batches: one LP per CTA ---------------------------------------------


int max_cluster_team()
{
        static int cached = 0;
        if (cached)
                return cached;
        const void * fn = kernel_alm_cluster(false);
        cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        for (int q = 16; q >= 2; q /= 2) {
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(q);
                cfg.blockDim = dim3(kBatchThreads);
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = q;
                attr[0].val.clusterDim.y = 1;
                attr[0].val.clusterDim.z = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                int clusters = 0;
                if (cudaOccupancyMaxActiveClusters(&clusters, fn, &cfg) == cudaSuccess
                    && clusters > 0) {
                        cached = q;
                        return q;
                }
                cudaGetLastError();
        }
        cached = 1;
        return 1;
}

struct AlmLaunch::Impl {
        AlmKernelArgs k;
};

AlmLaunch::AlmLaunch() : impl(new Impl) {}
AlmLaunch::~AlmLaunch()
{
        if (done)
                cudaEventDestroy(done);
        delete impl;
}

int alm_launch_async(DevInstance & d, const HostVectors & hv, size_t niter, double * x,
                     double * lam, const AlmSettings & s, const DeviceLayout * lay,
                     AlmLaunch & h, int team)
{
        if (team < 1 || team > 16) {
                set_error(ACDALM_EINVAL, "team of %d CTAs (1..16)", team);
                return ACDALM_EINVAL;
        }
        int r = alm_prepare(d, hv, niter, x, lam, false, s, lay, h.impl->k);
        if (r)
                return r;
        if (!h.done)
                ACD_CUDA_TRY(cudaEventCreateWithFlags(&h.done, cudaEventDisableTiming),
                             ACDALM_ECUDA);
        if (team == 1) {
                void * params[1] = {&h.impl->k};
                ACD_CUDA_TRY(cudaLaunchKernel(kernel_alm_single(g_exact), dim3(1),
                                              dim3(kBatchThreads), params, 0, d.stream),
                             ACDALM_ECUDA);
        } else {
                const void * fn = kernel_alm_cluster(g_exact);
                if (team > 8)
                        ACD_CUDA_TRY(cudaFuncSetAttribute(fn,
                                                          cudaFuncAttributeNonPortableClusterSizeAllowed,
                                                          1), ACDALM_ECUDA);
                cudaLaunchConfig_t cfg = {};
                cfg.gridDim = dim3(team);
                cfg.blockDim = dim3(kBatchThreads);
                cfg.dynamicSmemBytes = 0;
                cfg.stream = d.stream;
                cudaLaunchAttribute attr[1];
                attr[0].id = cudaLaunchAttributeClusterDimension;
                attr[0].val.clusterDim.x = team;
                attr[0].val.clusterDim.y = 1;
                attr[0].val.clusterDim.z = 1;
                cfg.attrs = attr;
                cfg.numAttrs = 1;
                void * params[1] = {&h.impl->k};
                ACD_CUDA_TRY(cudaLaunchKernelExC(&cfg, fn, params), ACDALM_ECUDA);
        }
        count_launch();
        ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaEventRecord(h.done, d.stream), ACDALM_ECUDA);
        return 0;
}

int alm_collect(DevInstance & d, AlmLaunch & h, double * x, double * lam, double * diag3,
                SolveStats & st)
{
        ACD_CUDA_TRY(cudaEventSynchronize(h.done), ACDALM_ECUDA);
        return alm_finish(d, h.impl->k, x, lam, nullptr, diag3, nullptr, nullptr, st, 0);
}

int run_alm_batch(std::vector<BatchEntry> & entries, size_t niter, double * seconds)
{
        int count = (int)entries.size();
        if (count == 0)
                return 0;
        std::vector<AlmKernelArgs> items(count);
        int r;
        for (int i = 0; i < count; i++) {
                BatchEntry & e = entries[i];
                if ((r = alm_prepare(*e.dev, e.hv, niter, e.x, e.lam, false, e.settings, e.lay,
                                     items[i])))
                        return r;
        }
        // largest LPs first: the persistent CTAs then balance the tail
        std::vector<int> order(count);
        for (int i = 0; i < count; i++)
                order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
                return entries[a].dev->nnz > entries[b].dev->nnz;
        });
        std::vector<AlmKernelArgs> sorted(count);
        for (int i = 0; i < count; i++)
                sorted[i] = items[order[i]];
        cudaStream_t s = entries[0].dev->stream;
        void * mem = nullptr;
        size_t bytes = sizeof(AlmKernelArgs) * count + 256;
        ACD_CUDA_TRY(cudaMallocAsync(&mem, bytes, s), ACDALM_ENOMEM);
        AlmKernelArgs * ditems = static_cast<AlmKernelArgs *>(mem);
        int * next = reinterpret_cast<int *>(static_cast<char *>(mem) + sizeof(AlmKernelArgs) * count);
        ACD_CUDA_TRY(cudaMemcpyAsync(ditems, sorted.data(), sizeof(AlmKernelArgs) * count,
                                     cudaMemcpyHostToDevice, s), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaMemsetAsync(next, 0, sizeof(int), s), ACDALM_ECUDA);
        const void * fn = kernel_alm_batch(g_exact);
        int dev = 0, sms = 0, per_sm = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBatchThreads, 0);
        int blocks = std::max(1, std::min(count, sms * std::max(per_sm, 1)));
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, s);
        {
                void * params[3] = {&ditems, &count, &next};
                ACD_CUDA_TRY(cudaLaunchKernel(fn, dim3(blocks), dim3(kBatchThreads), params, 0,
                                              s), ACDALM_ECUDA);
        }
        count_launch();
        ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        cudaEventRecord(e1, s);
        ACD_CUDA_TRY(cudaStreamSynchronize(s), ACDALM_ECUDA);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFreeAsync(mem, s);
        if (seconds)
                *seconds = ms * 1e-3;
        int worst = 0;
        for (int i = 0; i < count; i++) {
                BatchEntry & e = entries[i];
                e.ret = alm_finish(*e.dev, items[i], e.x, e.lam, nullptr, e.diag3, e.w_out,
                                   e.c_out, *e.stats, ms * 1e-3);
                if (e.ret < 0 && worst == 0)
                        worst = e.ret;
        }
        return worst;
}

static int run_inner(DevInstance & d, const HostVectors & hv, double * x,
                     size_t niter, double max_pg, double max_value,
                     double min_delta, FILE * log, size_t period, double * diag5,
                     double offset, SolveStats & st, bool mpg)
{
        int r = upload_problem(d, hv);
        if (r)
                return r;
        // step sizes of the uploaded instance (approx_update)
        step_size_kernel<<<std::max(1, std::min(4096, (d.n + 255) / 256)), 256, 0,
                           d.stream>>>(sell_at(d), d.w, d.beta, d.c0, d.v, d.inv_v);
        count_launch();
        ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        if ((r = upload_gather(d, d.x, x, d.col_orig, d.n, 0)) || (r = reset_ctl(d)))
                return r;
        ApproxKernelArgs k;
        memset(&k, 0, sizeof(k));
        k.P.m = d.m;
        k.P.n = d.n;
        k.P.A = sell_a(d);
        k.P.At = sell_at(d);
        k.P.b = d.b;
        k.P.w = d.w;
        k.P.c = d.c0;
        k.P.l = d.l;
        k.P.u = d.u;
        k.P.v = d.v;
        k.P.inv_v = d.inv_v;
        k.W = work_of(d);
        k.log = {d.log, d.log_cap, d.log_count};
        k.a.niter = (long long)std::min<size_t>(niter, (size_t)1 << 62);
        k.a.max_pg = max_pg;
        k.a.max_value = max_value;
        k.a.min_delta = min_delta;
        k.a.offset = offset;
        k.a.period = (long long)period;
        k.a.log = (log != nullptr);
        k.a.limit_ns = solve_limit_ns();
        k.x = d.x;
        k.ctl = static_cast<TeamCtl *>(d.ctl);
        k.slots = d.slots;
        k.result = d.result;
        k.out = static_cast<ApproxOut *>(d.out);
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        cudaEventRecord(e0, d.stream);
        const void * fn = mpg ? kernel_mpg_grid() : kernel_approx_grid(g_exact);
        if ((r = launch_coop(fn, d.grid_blocks, &k, d.slots, d.stream)))
                return r;
        cudaEventRecord(e1, d.stream);
        ACD_CUDA_TRY(cudaStreamSynchronize(d.stream), ACDALM_ECUDA);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        int status = 0;
        if ((r = read_status(d, status)))
                return r;
        ApproxOut out;
        ACD_CUDA_TRY(cudaMemcpy(&out, d.out, sizeof(out), cudaMemcpyDeviceToHost), ACDALM_ECUDA);
        fetch_logs(d, log);
        st.seconds = ms * 1e-3;
        st.inner = (unsigned long long)out.iters;
        st.status = status;
        if (status != 0) {
                set_error(status, "device solve failed with status %d (%s)", status,
                          status_text(status));
                return status;
        }
        if ((r = download_scatter(d, x, d.x, d.col_orig, d.n)))
                return r;
        if (diag5)
                for (int i = 0; i < 5; i++)
                        diag5[i] = out.diag[i];
        return out.reason;
}

size_t scratch_control_bytes(int max_blocks)
{
        return rounded(sizeof(TeamCtl)) + rounded(2 * (size_t)max_blocks * kSlotStride * 8)
                + rounded(2 * kRedMax * 8) + rounded(sizeof(ApproxOut)) + rounded(sizeof(int));
}

void carve_control(char * base, int max_blocks, ScratchSolve & s)
{
        char * p = base;
        s.max_blocks = max_blocks;
        s.ctl = carve<TeamCtl>(p, 1);
        s.slots = carve<double>(p, 2 * (size_t)max_blocks * kSlotStride);
        s.result = carve<double>(p, 2 * kRedMax);
        s.out = carve<ApproxOut>(p, 1);
        s.log_count = carve<int>(p, 1);
}

int run_approx_scratch(DevInstance & d, const HostVectors & hv, double * x_dev,
                       size_t niter, double max_pg, double max_value,
                       double min_delta, double * diag5, double offset,
                       const ScratchSolve & s, cudaStream_t stream)
{
        // the problem vectors go into the instance's own device arrays,
        // staged through its buffers (no allocation)
        int r = upload_problem(d, hv);
        if (r)
                return r;
        ACD_CUDA_TRY(cudaMemsetAsync(s.ctl, 0, sizeof(TeamCtl), stream), ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaMemsetAsync(s.log_count, 0, sizeof(int), stream), ACDALM_ECUDA);
        int nb = std::max(1, std::min(1024, (d.n + 255) / 256));
        step_size_kernel<<<nb, 256, 0, stream>>>(sell_at(d), d.w, d.beta, d.c0, s.v,
                                                 s.inv_v);
        count_launch();
        ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        if (d.n) {
                gather_kernel<<<nb, 256, 0, stream>>>(s.xd, x_dev, d.col_orig, d.n);
                count_launch();
                ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        }
        ApproxKernelArgs k;
        memset(&k, 0, sizeof(k));
        k.P.m = d.m;
        k.P.n = d.n;
        k.P.A = sell_a(d);
        k.P.At = sell_at(d);
        k.P.b = d.b;
        k.P.w = d.w;
        k.P.c = d.c0;
        k.P.l = d.l;
        k.P.u = d.u;
        k.P.v = s.v;
        k.P.inv_v = s.inv_v;
        InnerWork<double> W;
        W.zx = s.wn[0];
        W.zpx = s.wn[1];
        W.xx = s.wn[2];
        W.g = s.wn[3];
        W.g2 = s.wn[4];
        W.prev = s.wn[5];
        W.prev_alt = s.wn[6];
        W.alt_x = s.wn[7];
        W.ux = s.wn[8];
        W.vz = s.wm[0];
        W.vzp = s.wm[1];
        W.vx = s.wm[2];
        k.W = W;
        k.log = {nullptr, 0, s.log_count};
        k.a.niter = (long long)std::min<size_t>(niter, (size_t)1 << 62);
        k.a.max_pg = max_pg;
        k.a.max_value = max_value;
        k.a.min_delta = min_delta;
        k.a.offset = offset;
        k.a.period = 0;
        k.a.log = 0;
        k.a.limit_ns = solve_limit_ns();
        k.x = s.xd;
        k.ctl = static_cast<TeamCtl *>(s.ctl);
        k.slots = s.slots;
        k.result = s.result;
        k.out = static_cast<ApproxOut *>(s.out);
        const void * fn = kernel_approx_grid(g_exact);
        if ((r = launch_coop(fn, s.max_blocks, &k, s.slots, stream)))
                return r;
        if (d.n) {
                scatter_kernel<<<nb, 256, 0, stream>>>(x_dev, s.xd, d.col_orig, d.n);
                count_launch();
                ACD_CUDA_TRY(cudaGetLastError(), ACDALM_ECUDA);
        }
        int status = 0;
        ApproxOut out;
        ACD_CUDA_TRY(cudaMemcpyAsync(&status, &static_cast<TeamCtl *>(s.ctl)->status_w.v,
                                     sizeof(int), cudaMemcpyDeviceToHost, stream),
                     ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaMemcpyAsync(&out, s.out, sizeof(out), cudaMemcpyDeviceToHost, stream),
                     ACDALM_ECUDA);
        ACD_CUDA_TRY(cudaStreamSynchronize(stream), ACDALM_ECUDA);
        if (status != 0) {
                set_error(status, "device solve failed with status %d (%s)", status,
                          status_text(status));
                return status;
        }
        if (diag5)
                for (int i = 0; i < 5; i++)
                        diag5[i] = out.diag[i];
        return out.reason;
}

int run_approx(DevInstance & d, const HostVectors & hv, double * x,
               size_t niter, double max_pg, double max_value, double min_delta,
               FILE * log, size_t period, double * diag5, double offset,
               SolveStats & st)
{
        return run_inner(d, hv, x, niter, max_pg, max_value, min_delta, log, period,
                         diag5, offset, st, false);
}

int run_mpg(DevInstance & d, const HostVectors & hv, double * x, size_t niter,
            double max_pg, double max_value, FILE * log, size_t period,
            double * diag5, double offset, SolveStats & st)
{
        return run_inner(d, hv, x, niter, max_pg, max_value, 0, log, period, diag5,
                         offset, st, true);
}

}  // namespace acd

namespace acd {

// Loads every solver kernel now.  With lazy module loading the first launch
// of a kernel can wait for all kernels already running on the device, which
// would stall a server behind its longest solve.
void preload_solver_kernels()
{
        cudaFuncAttributes a;
        cudaFuncGetAttributes(&a, gather_kernel);
        cudaFuncGetAttributes(&a, scatter_kernel);
        cudaFuncGetAttributes(&a, step_size_kernel);
        for (int e = 0; e < 2; e++) {
                cudaFuncGetAttributes(&a, kernel_alm_grid(e));
                cudaFuncGetAttributes(&a, kernel_approx_grid(e));
                cudaFuncGetAttributes(&a, kernel_alm_batch(e));
                cudaFuncGetAttributes(&a, kernel_alm_single(e));
                cudaFuncGetAttributes(&a, kernel_alm_cluster(e));
        }
        cudaFuncGetAttributes(&a, kernel_mpg_grid());
        cudaFuncGetAttributes(&a, kernel_alm_grid_trace());
}

}  // namespace acd

extern "C" int acdalm_set_rounding(int exact)
{
        int old = acd::g_exact ? 1 : 0;
        acd::g_exact = exact != 0;
        return old;
}
