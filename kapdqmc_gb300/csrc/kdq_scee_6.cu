// Coupled SCEE (t-U, t-V, t-UV) / disorder-operator sweep kernels for lattice-size class MAXRM = 6.
#include "kdq_scee.cuh"

namespace kdq {
namespace {
template <int KIND, class T, class KT>
cudaError_t go(const SweepParams& P, int mode, int k, int npairs, size_t dyn, cudaStream_t st) {
  static size_t allowed = 0;   // dynamic shared memory the kernel was opened to
  if (dyn > allowed) {
    cudaError_t e = cudaFuncSetAttribute(k_scee<6, KIND, T, KT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
    allowed = dyn;
  }
  k_scee<6, KIND, T, KT><<<npairs, KDQ_THREADS, dyn, st>>>(P, mode, k);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_scee_rm6(const SweepParams& P, int mode, int k, int kind, bool kc, bool gc, int npairs,
                            size_t dyn, cudaStream_t st) {
  if (kind == KDQ_TV) return go<KDQ_TV, double, double>(P, mode, k, npairs, dyn, st);
  if (kind == KDQ_TUV)
    return gc ? go<KDQ_TUV, cd, double>(P, mode, k, npairs, dyn, st) : go<KDQ_TUV, double, double>(P, mode, k, npairs, dyn, st);
  return kc ? go<KDQ_TU, cd, cd>(P, mode, k, npairs, dyn, st) : go<KDQ_TU, cd, double>(P, mode, k, npairs, dyn, st);
}
}  // namespace kdq
