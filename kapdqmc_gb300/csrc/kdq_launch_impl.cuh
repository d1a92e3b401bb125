// Launcher templates: model x arithmetic x size class, instantiated by one
// translation unit per (model, precision) so they compile in parallel.
#pragma once
#include "kdq_launch.h"
#include "kdq_sweep.cuh"

namespace kdq {

template <int KIND, class T, class KT, int R, bool MIXED>
cudaError_t go(const SweepParams& P, int mode, int k, int nch, size_t dyn, cudaStream_t st) {
  k_block<KIND, T, KT, R, MIXED><<<nch, KDQ_THREADS, dyn, st>>>(P, mode, k);
  return cudaGetLastError();
}

template <int KIND, class T, class KT, bool MIXED>
cudaError_t go_rm(const SweepParams& P, int mode, int k, int maxrm, int nch, size_t dyn, cudaStream_t st) {
  if (maxrm == 1) return go<KIND, T, KT, 1, MIXED>(P, mode, k, nch, dyn, st);
  if (maxrm == 3) return go<KIND, T, KT, 3, MIXED>(P, mode, k, nch, dyn, st);
  return go<KIND, T, KT, 6, MIXED>(P, mode, k, nch, dyn, st);
}

// t-U: complex sweep, real or complex kinetic matrices
template <bool MIXED>
cudaError_t launch_tu_impl(const SweepParams& P, int mode, int k, int maxrm, bool kc, int nch, size_t dyn,
                           cudaStream_t st) {
  if (kc) return go_rm<KDQ_TU, cd, cd, MIXED>(P, mode, k, maxrm, nch, dyn, st);
  return go_rm<KDQ_TU, cd, double, MIXED>(P, mode, k, maxrm, nch, dyn, st);
}

template <bool MIXED>
cudaError_t prepare_tu_impl(size_t dyn) {
  const int b = (int)dyn;
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(k_block<KDQ_TU, cd, cd, 1, MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, b)) ||
      (e = cudaFuncSetAttribute(k_block<KDQ_TU, cd, cd, 3, MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, b)) ||
      (e = cudaFuncSetAttribute(k_block<KDQ_TU, cd, cd, 6, MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, b)) ||
      (e = cudaFuncSetAttribute(k_block<KDQ_TU, cd, double, 1, MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, b)) ||
      (e = cudaFuncSetAttribute(k_block<KDQ_TU, cd, double, 3, MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, b)) ||
      (e = cudaFuncSetAttribute(k_block<KDQ_TU, cd, double, 6, MIXED>, cudaFuncAttributeMaxDynamicSharedMemorySize, b)))
    return e;
  return cudaSuccess;
}

// t-V: real sweep with 2x2 bond rotations
template <bool MIXED>
cudaError_t launch_tv_impl(const SweepParams& P, int mode, int k, int maxrm, int nch, size_t dyn,
                           cudaStream_t st) {
  return go_rm<KDQ_TV, double, double, MIXED>(P, mode, k, maxrm, nch, dyn, st);
}

// t-U-V: complex sweep for U > 0, real otherwise
template <bool MIXED>
cudaError_t launch_tuv_impl(const SweepParams& P, int mode, int k, int maxrm, bool gc, int nch, size_t dyn,
                            cudaStream_t st) {
  if (gc) return go_rm<KDQ_TUV, cd, double, MIXED>(P, mode, k, maxrm, nch, dyn, st);
  return go_rm<KDQ_TUV, double, double, MIXED>(P, mode, k, maxrm, nch, dyn, st);
}

}  // namespace kdq
