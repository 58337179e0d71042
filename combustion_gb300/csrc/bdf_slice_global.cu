// The batched reactors' slice kernels with workspaces and factorisations in global memory (FP64 and mixed-precision first
// Newton iterations), instantiated in a translation unit of their own so that the variants compile in
// parallel.
#include "bdf_device.cuh"

namespace cbg {
namespace bdf {

SliceFn slice_kernel_global_fn(bool mixed) { return mixed ? slice_kernel_global<true> : slice_kernel_global<false>; }

}  // namespace bdf
}  // namespace cbg
