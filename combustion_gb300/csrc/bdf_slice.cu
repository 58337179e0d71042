// The batched reactors' slice kernels with workspaces in shared memory (FP64 and mixed-precision first
// Newton iterations), instantiated in a translation unit of their own so that the variants compile in
// parallel.
#include "bdf_device.cuh"

namespace cbg {
namespace bdf {

SliceFn slice_kernel_fn(bool mixed) { return mixed ? slice_kernel<true> : slice_kernel<false>; }

}  // namespace bdf
}  // namespace cbg
