// Coupled incremental SCEE sweep kernels (t-U), FP64.
#include "kdq_launch.h"
#include "kdq_scee.cuh"

namespace kdq {
namespace {
template <class KT, int R>
cudaError_t go_scee(const SweepParams& P, int mode, int k, int npairs, size_t dyn, cudaStream_t st) {
  static size_t allowed = 0;   // dynamic shared memory the kernel was opened to
  if (dyn > allowed) {
    cudaError_t e = cudaFuncSetAttribute(k_scee<R, cd, KT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
    allowed = dyn;
  }
  k_scee<R, cd, KT><<<npairs, KDQ_THREADS, dyn, st>>>(P, mode, k);
  return cudaGetLastError();
}
}  // namespace

size_t scee_dyn_bytes(int Ns) { return scee_tape_bytes(Ns) + sizeof(SceeSmem<cd>); }

cudaError_t launch_scee(const SweepParams& P, int mode, int k, int maxrm, bool kc, int npairs, cudaStream_t st) {
  const size_t dyn = scee_dyn_bytes(P.Ns);
  if (kc) {
    if (maxrm == 1) return go_scee<cd, 1>(P, mode, k, npairs, dyn, st);
    if (maxrm == 3) return go_scee<cd, 3>(P, mode, k, npairs, dyn, st);
    return go_scee<cd, 6>(P, mode, k, npairs, dyn, st);
  }
  if (maxrm == 1) return go_scee<double, 1>(P, mode, k, npairs, dyn, st);
  if (maxrm == 3) return go_scee<double, 3>(P, mode, k, npairs, dyn, st);
  return go_scee<double, 6>(P, mode, k, npairs, dyn, st);
}
}  // namespace kdq
