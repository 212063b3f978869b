// Compiles ALM solves on one CTA per LP, the reference's separate rounding.
#include "kernels.cuh"

namespace acd {

const void * kernel_alm_single_exact() { return (const void *)alm_single_kernel<true>; }
const void * kernel_alm_batch_exact() { return (const void *)alm_batch_kernel<true>; }

}  // namespace acd
