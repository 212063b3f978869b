// Compiles ALM solves on one thread-block cluster per LP (large served LPs).
#include "kernels.cuh"

namespace acd {

const void * kernel_alm_cluster(bool exact)
{
        return exact ? (const void *)alm_cluster_kernel<true>
                     : (const void *)alm_cluster_kernel<false>;
}

}  // namespace acd
