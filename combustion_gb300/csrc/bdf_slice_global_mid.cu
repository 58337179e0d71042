// The batched reactors' slice kernels with workspaces in global memory and 80 registers a thread (three
// 256-thread blocks per SM), in a translation unit of their own so that the variants compile in parallel.
#include "bdf_device.cuh"

namespace cbg {
namespace bdf {

SliceFn slice_kernel_global_mid_fn(bool mixed) {
    return mixed ? slice_kernel_global_mid<true> : slice_kernel_global_mid<false>;
}

}  // namespace bdf
}  // namespace cbg
