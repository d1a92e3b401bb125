// t-U model kernels: complex sweep, real or complex kinetic matrices.
#include "kdq_launch.h"
#include "kdq_sweep.cuh"

namespace kdq {
template <class KT, int R>
static cudaError_t go(const SweepParams& P, int mode, int k, int nch, size_t dyn, cudaStream_t st) {
  k_block<KDQ_TU, cd, KT, R><<<nch, KDQ_THREADS, dyn, st>>>(P, mode, k);
  return cudaGetLastError();
}
cudaError_t launch_tu(const SweepParams& P, int mode, int k, int maxrm, bool kc, int nch, size_t dyn,
                      cudaStream_t st) {
  if (kc) {
    if (maxrm == 1) return go<cd, 1>(P, mode, k, nch, dyn, st);
    if (maxrm == 3) return go<cd, 3>(P, mode, k, nch, dyn, st);
    return go<cd, 6>(P, mode, k, nch, dyn, st);
  }
  if (maxrm == 1) return go<double, 1>(P, mode, k, nch, dyn, st);
  if (maxrm == 3) return go<double, 3>(P, mode, k, nch, dyn, st);
  return go<double, 6>(P, mode, k, nch, dyn, st);
}
}  // namespace kdq
