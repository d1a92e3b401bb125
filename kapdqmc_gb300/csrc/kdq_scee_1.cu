// Coupled SCEE sweep kernels for lattice-size class MAXRM = 1.
#include "kdq_scee.cuh"

namespace kdq {
namespace {
template <class KT>
cudaError_t go(const SweepParams& P, int mode, int k, int npairs, size_t dyn, cudaStream_t st) {
  static size_t allowed = 0;   // dynamic shared memory the kernel was opened to
  if (dyn > allowed) {
    cudaError_t e = cudaFuncSetAttribute(k_scee<1, cd, KT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
    allowed = dyn;
  }
  k_scee<1, cd, KT><<<npairs, KDQ_THREADS, dyn, st>>>(P, mode, k);
  return cudaGetLastError();
}
}  // namespace

cudaError_t launch_scee_rm1(const SweepParams& P, int mode, int k, bool kc, int npairs, size_t dyn, cudaStream_t st) {
  return kc ? go<cd>(P, mode, k, npairs, dyn, st) : go<double>(P, mode, k, npairs, dyn, st);
}
}  // namespace kdq
