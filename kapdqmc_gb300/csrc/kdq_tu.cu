// tu model sweep kernels, FP64.
#include "kdq_launch_impl.cuh"

namespace kdq {
cudaError_t launch_tu(const SweepParams& P, int mode, int k, int maxrm, bool kc, int nch, size_t dyn, cudaStream_t st) {
  return launch_tu_impl<false>(P, mode, k, maxrm, kc, nch, dyn, st);
}
cudaError_t prepare_tu(size_t dyn) { return prepare_tu_impl<false>(dyn); }
}  // namespace kdq
