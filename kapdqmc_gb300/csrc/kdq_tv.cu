// tv model sweep kernels, FP64.
#include "kdq_launch_impl.cuh"

namespace kdq {
cudaError_t launch_tv(const SweepParams& P, int mode, int k, int maxrm, int nch, size_t dyn, cudaStream_t st) {
  return launch_tv_impl<false>(P, mode, k, maxrm, nch, dyn, st);
}
}  // namespace kdq
