// Allocation-free Grover determinant: kdq_grover_det_noalloc.
//
// Some callers cannot call cudaMalloc: code that records work into a CUDA
// graph or must not stall (cudaMalloc may synchronize the device), and
// processes whose free device memory is already reserved by another
// allocator (a framework's caching pool), where a fresh cudaMalloc can fail.
// This entry point runs the same Grover kernel as kdq_grover_det, but every
// byte of its scratch comes from the fixed device array below, so the call
// allocates nothing: the caller passes device buffers for the inputs and the
// output and the library only launches kernels on the caller's stream.
//
// The array is KDQ_NOALLOC_GROVER_BYTES (8 MiB) in every GPU that loads the
// library, for the life of the process.  All calls share it and it keeps the
// previous call's contents; the kernels overwrite everything they read
// except the index-error flag, which each call clears first.  Calls that
// overlap on the GPU (different streams, or different host threads without
// ordering) race on the array and must be serialised by the caller.
#include <mutex>
#include <string>

#include "kdq_launch.h"

#define KDQ_NOALLOC_GROVER_BYTES (8u << 20)
#define KDQ_NOALLOC_MAX_DEVICES 64

namespace {

// Scratch of kdq_grover_det_noalloc: [index flag + 0-based region sites]
// [pivots][gathered blocks and Grover matrices], each part 256-byte aligned.
static __device__ __align__(256) unsigned char g_grover_scratch[KDQ_NOALLOC_GROVER_BYTES];

std::mutex g_mu;
void* g_scratch_addr[KDQ_NOALLOC_MAX_DEVICES] = {};

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Device address of the scratch array for the current device.  Host code
// cannot use the array's name as a device pointer, so the address comes from
// cudaGetSymbolAddress with the device current.  It is looked up again on
// every call whose stream is not capturing (cudaDeviceReset reloads the
// module, and the array may then sit at another address); while a stream
// captures, the address from the device's last uncaptured call is used, so
// the first call on a device has to come before any capture.
cudaError_t scratch_for_current_device(cudaStream_t st, void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= KDQ_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  e = cudaStreamIsCapturing(st, &cap);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lk(g_mu);
  if (cap == cudaStreamCaptureStatusNone) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_grover_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_addr[dev] = p;
  } else if (!g_scratch_addr[dev]) {
    return cudaErrorStreamCaptureUnsupported;
  }
  *out = g_scratch_addr[dev];
  return cudaSuccess;
}

// 1-based caller indices -> 0-based, clamped into range; an out-of-range
// index raises the flag (cleared here first) instead of being dereferenced.
__global__ void k_region_index(const int32_t* index1, int nA, int Ns, int* flag, int* index0) {
  if (threadIdx.x == 0) *flag = 0;
  __syncthreads();
  for (int i = threadIdx.x; i < nA; i += blockDim.x) {
    const int v = index1[i] - 1;
    const bool ok = v >= 0 && v < Ns;
    if (!ok) atomicOr(flag, 1);
    index0[i] = ok ? v : 0;
  }
}

// Determinants of a call with an invalid region become NaN.
__global__ void k_poison(const int* flag, double* det, int npairs) {
  if (*flag == 0) return;
  for (int i = threadIdx.x; i < 2 * npairs; i += blockDim.x) det[i] = __longlong_as_double(0x7ff8000000000000LL);
}

}  // namespace

namespace kdq {
void set_global_error(const std::string& msg);
}

extern "C" int kdq_grover_det_noalloc(const double* G, int32_t Ns, int32_t g_complex, int32_t npairs,
                                      const int32_t* index, int32_t nA, double* det, void* stream) {
  if (!G || !index || !det) {
    kdq::set_global_error("kdq_grover_det_noalloc: NULL device pointer");
    return KDQ_ERR_ARG;
  }
  if (Ns < 1 || nA < 1 || nA > Ns || npairs < 0) {
    kdq::set_global_error("kdq_grover_det_noalloc: need 1 <= nA <= Ns and npairs >= 0");
    return KDQ_ERR_ARG;
  }
  if (npairs == 0) return KDQ_OK;
  const size_t head = align256(sizeof(int) * (1 + (size_t)nA));
  const size_t pivs = align256(sizeof(int) * (size_t)npairs * nA);
  const size_t need = head + pivs + kdq::grover_scratch_bytes(nA, npairs, g_complex != 0);
  if (need > KDQ_NOALLOC_GROVER_BYTES) {
    kdq::set_global_error("kdq_grover_det_noalloc: " + std::to_string(npairs) + " pairs with a region of " +
                          std::to_string(nA) + " sites need " + std::to_string(need) +
                          " bytes of scratch; the fixed maximum is " + std::to_string(KDQ_NOALLOC_GROVER_BYTES) +
                          " bytes (use fewer pairs per call)");
    return KDQ_ERR_ARG;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  void* base = nullptr;
  cudaError_t e = scratch_for_current_device(st, &base);
  if (e != cudaSuccess) {
    kdq::set_global_error(std::string("kdq_grover_det_noalloc: scratch address: ") + cudaGetErrorString(e));
    return KDQ_ERR_CUDA;
  }
  unsigned char* b = static_cast<unsigned char*>(base);
  int* flag = reinterpret_cast<int*>(b);
  int* index0 = flag + 1;
  int* piv = reinterpret_cast<int*>(b + head);
  void* blocks = b + head + pivs;
  k_region_index<<<1, 256, 0, st>>>(index, nA, Ns, flag, index0);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = kdq::launch_grover(G, Ns, g_complex != 0, index0, nA, npairs, blocks, piv, det, st);
  if (e == cudaSuccess) {
    k_poison<<<1, 256, 0, st>>>(flag, det, npairs);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) {
    kdq::set_global_error(std::string("kdq_grover_det_noalloc: launch: ") + cudaGetErrorString(e));
    return KDQ_ERR_CUDA;
  }
  return KDQ_OK;
}
