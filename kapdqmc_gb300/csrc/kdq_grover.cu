// Grover-determinant kernels and the handle-free C entry point.
#include <string>

#include "kdq_grover.cuh"
#include "kdq_launch.h"

namespace kdq {
cudaError_t launch_grover(const void* G, int Ns, bool gc, const int* index, int nA, int npairs, void* scratch,
                          int* pivs, double* det, cudaStream_t st) {
  if (npairs <= 0) return cudaSuccess;
  if (gc)
    k_grover<cd><<<npairs, 256, 0, st>>>(static_cast<const cd*>(G), Ns, index, nA, npairs,
                                         static_cast<cd*>(scratch), pivs, det);
  else
    k_grover<double><<<npairs, 256, 0, st>>>(static_cast<const double*>(G), Ns, index, nA, npairs,
                                             static_cast<double*>(scratch), pivs, det);
  return cudaGetLastError();
}
}  // namespace kdq
