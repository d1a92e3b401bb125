// t-V model kernels: real sweep with 2x2 bond rotations.
#include "kdq_launch.h"
#include "kdq_sweep.cuh"

namespace kdq {
template <int R>
static cudaError_t go(const SweepParams& P, int mode, int k, int nch, size_t dyn, cudaStream_t st) {
  k_block<KDQ_TV, double, double, R><<<nch, KDQ_THREADS, dyn, st>>>(P, mode, k);
  return cudaGetLastError();
}
cudaError_t launch_tv(const SweepParams& P, int mode, int k, int maxrm, int nch, size_t dyn, cudaStream_t st) {
  if (maxrm == 1) return go<1>(P, mode, k, nch, dyn, st);
  if (maxrm == 3) return go<3>(P, mode, k, nch, dyn, st);
  return go<6>(P, mode, k, nch, dyn, st);
}
}  // namespace kdq
