// Compiles ALM solves on one CTA per LP (batches, small served LPs), fused
// multiply-adds.
#include "kernels.cuh"

namespace acd {

const void * kernel_alm_single_fast() { return (const void *)alm_single_kernel<false>; }
const void * kernel_alm_batch_fast() { return (const void *)alm_batch_kernel<false>; }

}  // namespace acd
