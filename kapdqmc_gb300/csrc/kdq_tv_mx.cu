// tv model sweep kernels, mixed precision.
#include "kdq_launch_impl.cuh"

namespace kdq {
cudaError_t launch_tv_mixed(const SweepParams& P, int mode, int k, int maxrm, int nch, size_t dyn, cudaStream_t st) {
  return launch_tv_impl<true>(P, mode, k, maxrm, nch, dyn, st);
}
}  // namespace kdq
