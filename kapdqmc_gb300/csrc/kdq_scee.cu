// Coupled incremental SCEE sweep kernels (t-U), FP64: dispatch.  The kernel
// instantiations live in kdq_scee_1.cu, kdq_scee_3.cu, kdq_scee_6.cu (one
// lattice-size class each, compiled in parallel).
#include "kdq_launch.h"
#include "kdq_scee.cuh"

namespace kdq {
cudaError_t launch_scee_rm1(const SweepParams& P, int mode, int k, int kind, bool kc, bool gc, int npairs,
                            size_t dyn, cudaStream_t st);
cudaError_t launch_scee_rm3(const SweepParams& P, int mode, int k, int kind, bool kc, bool gc, int npairs,
                            size_t dyn, cudaStream_t st);
cudaError_t launch_scee_rm6(const SweepParams& P, int mode, int k, int kind, bool kc, bool gc, int npairs,
                            size_t dyn, cudaStream_t st);

size_t scee_dyn_bytes(int Ns, int kind) {
  if (kind == KDQ_TU) return scee_tape_bytes(Ns) + sizeof(SceeSmem<cd>);
  return scee_tape_bytes(Ns) + sizeof(SceeSmem2<cd>);   // the larger of the two rank-2 variants
}

cudaError_t launch_scee(const SweepParams& P, int mode, int k, int maxrm, bool kc, bool gc, int npairs,
                        cudaStream_t st) {
  const size_t dyn = scee_dyn_bytes(P.Ns, P.kind);
  if (maxrm == 1) return launch_scee_rm1(P, mode, k, P.kind, kc, gc, npairs, dyn, st);
  if (maxrm == 3) return launch_scee_rm3(P, mode, k, P.kind, kc, gc, npairs, dyn, st);
  return launch_scee_rm6(P, mode, k, P.kind, kc, gc, npairs, dyn, st);
}
}  // namespace kdq
