// Shared host-side definitions for libacdalm: status codes, error reporting,
// CUDA error checks.
#pragma once
#include <cstddef>
#include <cstdint>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "../../include/acdalm_ext.h"

namespace acd {

// A named host-side range for NVTX-aware profilers (upload, solve kernel,
// download, ...); costs nothing when no profiler is attached.
struct NvtxRange {
        explicit NvtxRange(const char * name) { nvtxRangePushA(name); }
        ~NvtxRange() { nvtxRangePop(); }
        NvtxRange(const NvtxRange &) = delete;
        NvtxRange & operator=(const NvtxRange &) = delete;
};

// Records the last error of the calling thread (read back through
// acdalm_last_error) and, unless ACDALM_QUIET is set, prints it to stderr.
void set_error(int code, const char * fmt, ...);
int last_error_code();

// True when a CUDA device is usable; sets an error message otherwise.
bool device_ready();

// Counts every kernel launch the library makes (acdalm_launch_count).
void count_launch(unsigned n = 1);

}  // namespace acd

#define ACD_CUDA_TRY(call, ret)                                              \
        do {                                                                 \
                cudaError_t acd_err_ = (call);                               \
                if (acd_err_ != cudaSuccess) {                               \
                        ::acd::set_error(ACDALM_ECUDA, "%s:%d: %s: %s",      \
                                         __FILE__, __LINE__, #call,          \
                                         cudaGetErrorString(acd_err_));      \
                        return ret;                                          \
                }                                                            \
        } while (0)
