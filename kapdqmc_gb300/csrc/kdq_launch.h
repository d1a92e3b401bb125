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
}  // namespace kdq
