// tu model sweep kernels, mixed precision.
#include "kdq_launch_impl.cuh"

namespace kdq {
cudaError_t launch_tu_mixed(const SweepParams& P, int mode, int k, int maxrm, bool kc, int nch, size_t dyn, cudaStream_t st) {
  return launch_tu_impl<true>(P, mode, k, maxrm, kc, nch, dyn, st);
}
cudaError_t prepare_tu_mixed(size_t dyn) { return prepare_tu_impl<true>(dyn); }
}  // namespace kdq
