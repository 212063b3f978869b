// approx_solve_static: the APPROX solve for callers that cannot allocate
// device memory at solve time.
//
// Some callers of this library cannot call cudaMalloc when they solve:
// frameworks whose caching allocator has already taken the device memory
// budget (a cudaMalloc beside it fails or fragments what it holds), and
// latency-bound loops that cannot take cudaMalloc's implicit device-wide
// synchronisation, which stalls every other stream.  This entry point uses
// no memory beyond its inputs and outputs except one fixed array declared
// below, which every GPU that loads the library holds until the process
// exits.  Every call shares that array, so calls that overlap on the GPU
// (from other threads or streams) race.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/acdalm_ext.h"
#include "common.h"
#include "instance.h"
#include "objects.h"

namespace {

// All solver scratch of approx_solve_static: control words, reduction slots
// for up to kStaticBlocks CTAs, the output block, the step sizes, x in
// device order and the APPROX workspace (12 vectors of n and 6 of m
// doubles).
constexpr size_t kStaticScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr int kStaticBlocks = 1024;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_lock;
void * g_scratch_addr[kMaxDevices] = {};

size_t rounded(size_t bytes)
{
        return (bytes + 255) & ~size_t(255);
}

size_t scratch_bytes_needed(size_t n, size_t m)
{
        return acd::scratch_control_bytes(kStaticBlocks) + 12 * rounded(n * 8)
                + 3 * rounded(m * 16);
}

// The device address of g_static_scratch on the current device, looked up
// once per device with that device current.  In host code the name
// g_static_scratch is only a host-side stand-in, never a device address.
int scratch_address(void ** out)
{
        int dev = 0;
        ACD_CUDA_TRY(cudaGetDevice(&dev), ACDALM_ECUDA);
        if (dev < 0 || dev >= kMaxDevices) {
                acd::set_error(ACDALM_EINVAL, "approx_solve_static: device %d", dev);
                return ACDALM_EINVAL;
        }
        std::lock_guard<std::mutex> g(g_lock);
        if (!g_scratch_addr[dev]) {
                void * p = nullptr;
                cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
                if (e != cudaSuccess || p == nullptr) {
                        acd::set_error(ACDALM_ECUDA,
                                       "approx_solve_static: cudaGetSymbolAddress: %s",
                                       cudaGetErrorString(e));
                        return ACDALM_ECUDA;
                }
                g_scratch_addr[dev] = p;
        }
        *out = g_scratch_addr[dev];
        return 0;
}

}  // namespace

extern "C" int approx_solve_static(double * x, size_t n, approx_t * approx,
                                   size_t niter, double max_pg, double max_value,
                                   double min_delta, double * OUT_diagnosis,
                                   double offset, void * stream)
{
        if (!approx || n != approx->nvars || (n && !x)) {
                acd::set_error(ACDALM_EINVAL,
                               "approx_solve_static: n does not match the instance");
                return ACDALM_EINVAL;
        }
        size_t need = scratch_bytes_needed(approx->nvars, approx->nrhs);
        if (need > kStaticScratchBytes) {
                acd::set_error(ACDALM_EINVAL,
                               "approx_solve_static: an instance with %zu columns and %zu "
                               "rows needs %zu bytes of solver scratch; the fixed array "
                               "holds %zu (about 12 n + 6 m <= 4.17 million doubles)",
                               approx->nvars, approx->nrhs, need, kStaticScratchBytes);
                return ACDALM_EINVAL;
        }
        std::lock_guard<std::mutex> g(approx->lock);
        if (!approx->dev_ready) {
                acd::set_error(ACDALM_EINVAL,
                               "approx_solve_static: the instance has no device copy yet; "
                               "call approx_solve (or mpg_solve / cd_solve) on it once "
                               "first, outside any stream capture");
                return ACDALM_EINVAL;
        }
        if (!acd::device_ready())
                return ACDALM_ENODEV;
        void * base = nullptr;
        int r = scratch_address(&base);
        if (r)
                return r;
        char * p = static_cast<char *>(base);
        auto carve = [&](size_t bytes) {
                char * q = p;
                p += rounded(bytes);
                return q;
        };
        acd::ScratchSolve s;
        acd::carve_control(carve(acd::scratch_control_bytes(kStaticBlocks)), kStaticBlocks, s);
        s.v = reinterpret_cast<double *>(carve(n * 8));
        s.inv_v = reinterpret_cast<double *>(carve(n * 8));
        s.xd = reinterpret_cast<double *>(carve(n * 8));
        for (auto & w : s.wn)
                w = reinterpret_cast<double *>(carve(n * 8));
        for (auto & w : s.wm)
                w = reinterpret_cast<double *>(carve(approx->nrhs * 16));
        acd::HostVectors hv;
        hv.b = approx->s_rhs.data();
        hv.w = approx->s_weight.data();
        hv.c0 = approx->s_linear.data();
        hv.l = approx->s_lower.data();
        hv.u = approx->s_upper.data();
        return acd::run_approx_scratch(approx->dev, hv, x, niter, max_pg, max_value,
                                       min_delta, OUT_diagnosis, offset, s,
                                       static_cast<cudaStream_t>(stream));
}
