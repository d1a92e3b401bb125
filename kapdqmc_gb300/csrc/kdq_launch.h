// Per-model kernel launchers (one translation unit per model so the three
// are compiled in parallel).
#pragma once
#include <cuda_runtime.h>

#include "kdq_params.h"

namespace kdq {
// maxrm: row groups of 32 per lane in the block GEMM (1, 3 or 6).
cudaError_t launch_tu(const SweepParams& P, int mode, int k, int maxrm, bool k_complex,
                      int nchains, size_t dyn, cudaStream_t st);
cudaError_t launch_tv(const SweepParams& P, int mode, int k, int maxrm, int nchains, size_t dyn,
                      cudaStream_t st);
cudaError_t launch_tuv(const SweepParams& P, int mode, int k, int maxrm, bool g_complex,
                       int nchains, size_t dyn, cudaStream_t st);
// the same in mixed precision (FP32 working type, double-float stabilisation)
cudaError_t launch_tu_mixed(const SweepParams& P, int mode, int k, int maxrm, bool k_complex,
                            int nchains, size_t dyn, cudaStream_t st);
cudaError_t launch_tv_mixed(const SweepParams& P, int mode, int k, int maxrm, int nchains, size_t dyn,
                            cudaStream_t st);
cudaError_t launch_tuv_mixed(const SweepParams& P, int mode, int k, int maxrm, bool g_complex,
                             int nchains, size_t dyn, cudaStream_t st);
// Allow `dyn` bytes of dynamic shared memory for every t-U sweep kernel
// (the self-learning cluster moves need more than the default 48 KB).
cudaError_t prepare_tu(size_t dyn);
cudaError_t prepare_tu_mixed(size_t dyn);
// Coupled SCEE sweep (t-U, t-V, t-UV): one CTA per replica pair (chains 2p, 2p+1),
// or per chain for the disorder-operator sweep (t-U).
cudaError_t launch_scee(const SweepParams& P, int mode, int k, int maxrm, bool k_complex, bool g_complex,
                        int npairs, cudaStream_t st);
size_t scee_dyn_bytes(int Ns, int kind);
// Grover determinants of npairs replica pairs (matrices 2p, 2p+1 of G).
// scratch: npairs * 3 * nA^2 elements of the G type; pivs: npairs * nA.
cudaError_t launch_grover(const void* G, int Ns, bool g_complex, const int* index, int nA, int npairs,
                          void* scratch, int* pivs, double* det, cudaStream_t st);
size_t grover_scratch_bytes(int nA, int npairs, bool g_complex);
}  // namespace kdq
