// tuv model sweep kernels, mixed precision.
#include "kdq_launch_impl.cuh"

namespace kdq {
cudaError_t launch_tuv_mixed(const SweepParams& P, int mode, int k, int maxrm, bool gc, int nch, size_t dyn, cudaStream_t st) {
  return launch_tuv_impl<true>(P, mode, k, maxrm, gc, nch, dyn, st);
}
}  // namespace kdq
