// Error reporting and device selection.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "common.h"

namespace acd {

namespace {
thread_local char t_msg[512] = "";
thread_local int t_code = 0;
}  // namespace

void set_error(int code, const char * fmt, ...)
{
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(t_msg, sizeof(t_msg), fmt, ap);
        va_end(ap);
        t_code = code;
        const char * quiet = getenv("ACDALM_QUIET");
        if (!(quiet && quiet[0] == '1'))
                fprintf(stderr, "libacdalm: %s\n", t_msg);
}

static std::atomic<unsigned long long> g_launches{0};

void count_launch(unsigned n)
{
        g_launches.fetch_add(n, std::memory_order_relaxed);
}

unsigned long long launch_count()
{
        return g_launches.load();
}

int last_error_code()
{
        return t_code;
}

void preload_solver_kernels();
void preload_spmv_kernels();

bool device_ready()
{
        static int count = -1;
        static int device = 0;
        static bool loaded[64] = {};
        if (count < 0) {
                if (cudaGetDeviceCount(&count) != cudaSuccess)
                        count = 0;
                const char * d = getenv("ACDALM_DEVICE");
                device = d ? atoi(d) : 0;
        }
        if (count <= 0 || device >= count) {
                set_error(ACDALM_ENODEV, "no usable CUDA device (libacdalm runs its "
                          "solves and products on the GPU only)");
                return false;
        }
        if (cudaSetDevice(device) != cudaSuccess) {
                set_error(ACDALM_ENODEV, "cudaSetDevice(%d) failed", device);
                return false;
        }
        if (device < 64 && !loaded[device]) {
                static std::mutex mu;
                std::lock_guard<std::mutex> g(mu);
                if (!loaded[device]) {
                        preload_solver_kernels();
                        preload_spmv_kernels();
                        loaded[device] = true;
                }
        }
        return true;
}

}  // namespace acd

extern "C" const char * acdalm_last_error(void)
{
        return acd::t_msg;
}

extern "C" unsigned long long acdalm_launch_count(void)
{
        return acd::launch_count();
}

extern "C" int acdalm_take_error(void)
{
        int c = acd::t_code;
        acd::t_code = 0;
        acd::t_msg[0] = 0;
        return c;
}
