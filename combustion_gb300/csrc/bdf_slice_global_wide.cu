// The batched reactors' slice kernels with workspaces in global memory and 128 registers a thread (two
// 256-thread blocks per SM), in a translation unit of their own so that the variants compile in parallel.
#include "bdf_device.cuh"

namespace cbg {
namespace bdf {

SliceFn slice_kernel_global_wide_fn(bool mixed) {
    return mixed ? slice_kernel_global_wide<true> : slice_kernel_global_wide<false>;
}

}  // namespace bdf
}  // namespace cbg
