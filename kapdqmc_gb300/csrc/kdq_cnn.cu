// Training and inference kernels of the self-learning effective model
// (kdq_cnn.cuh) and their handle-free C entry points.
//
// A work item is one tile of R slices (rows) of one configuration (R picked
// per lattice and batch by timing, see autotune).  The
// forward kernel stages the tile's field window and layer-1 activations in
// shared memory and adds its share of F to the configuration's total.  The
// backward kernel is persistent (one CTA per SM): it recomputes the
// activations of each work item it takes, back-propagates dF through the
// layers in shared memory and keeps its parameter-gradient partials in
// registers until all items are done, so the global gradient receives one
// atomic add per parameter per CTA.
#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <numeric>
#include <tuple>
#include <random>
#include <string>
#include <vector>

#include "../../include/kapdqmc.h"
#include "kdq_cnn.cuh"

static_assert(KDQ_CNN_NPARAM == KDQ_CNN_PARAMS, "parameter count of the header and the kernels");

namespace kdq {
void set_global_error(const std::string& msg);
}

namespace {
using namespace kdq;

constexpr int CH = KDQ_CNN_CH;
constexpr size_t SMEM_MAX = 227 * 1024;

__device__ __forceinline__ int wrap1(int v, int n) {  // v in [-n, 2n)
  return v < 0 ? v + n : (v >= n ? v - n : v);
}

__host__ __device__ inline size_t align16(size_t b) { return (b + 15) & ~size_t(15); }

// Activation rows in shared memory are padded to an odd stride, so that the
// 16 channels of one site fall into 16 different banks.
__host__ __device__ inline int pad_stride(int Ns) { return Ns | 1; }

size_t fwd_smem(int R, int Ns) {
  const int Sp = pad_stride(Ns);
  return align16(sizeof(CnnW)) + align16((size_t)(R + 2) * CH * Sp * sizeof(float)) + align16((size_t)(R + 4) * Ns);
}
size_t bwd_smem(int R, int Ns) {
  const int Sp = pad_stride(Ns);
  return align16(sizeof(CnnW)) + align16((size_t)(R + 4) * CH * Sp * sizeof(float)) +
         align16((size_t)(R + 2) * CH * Sp * sizeof(float)) + align16((size_t)R * CH * Sp * sizeof(float)) +
         align16((size_t)(R + 6) * Ns) + 64 * sizeof(float);
}

// F[b] += share of tile blockIdx.x of configuration idx[b] (blockIdx.y = b).
__global__ void __launch_bounds__(256) k_cnn_fwd(const uint8_t* __restrict__ fields, const int* __restrict__ idx,
                                                 int Nt, int Ns, int R, const __nv_bfloat16* __restrict__ prm,
                                                 double* __restrict__ F) {
  extern __shared__ __align__(16) unsigned char smem[];
  CnnW& w = *reinterpret_cast<CnnW*>(smem);
  const int Sp = pad_stride(Ns);
  float* a1 = reinterpret_cast<float*>(smem + align16(sizeof(CnnW)));
  uint8_t* x = reinterpret_cast<uint8_t*>(a1) + align16((size_t)(R + 2) * CH * Sp * sizeof(float));
  __shared__ double red[32];
  const int b = blockIdx.y, r0 = blockIdx.x * R;
  const uint8_t* s = fields + (size_t)(idx ? idx[b] : b) * Nt * Ns;
  load_cnn_weights(w, prm);
  for (int e = threadIdx.x; e < (R + 4) * Ns; e += blockDim.x) {
    const int rr = e / Ns, j = e - rr * Ns;
    x[e] = s[(size_t)wrapi(r0 - 2 + rr, Nt) * Ns + j];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < (R + 2) * CH * Ns; e += blockDim.x) {
    const int j = e % Ns, o = (e / Ns) % CH, rr = e / (Ns * CH);
    a1[(rr * CH + o) * Sp + j] = cnn_a1(w, o, [&](int dt, int dj) { return (int)x[(rr + 1 + dt) * Ns + wrap1(j + dj, Ns)]; });
  }
  __syncthreads();
  double part = 0.0;
  for (int p = threadIdx.x; p < R * Ns; p += blockDim.x) {
    const int rr = p / Ns, j = p - rr * Ns;
    if (r0 + rr >= Nt) continue;
    float z[CH];
    cnn_z2(w, z, [&](int c, int dt, int dj) { return a1[((rr + 1 + dt) * CH + c) * Sp + wrap1(j + dj, Ns)]; });
    float v = w.b3;
#pragma unroll
    for (int o = 0; o < CH; ++o) v = fmaf(w.w3s[o], tanhf(z[o]), v);
    part += v;
  }
  // block sum
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
    atomicAdd(&F[b], t);
  }
}

// gradient of sum_b dF[b] F(s_b) with respect to every parameter, added to grad
__global__ void __launch_bounds__(256, 1) k_cnn_bwd(const uint8_t* __restrict__ fields, const int* __restrict__ idx,
                                                    int B, int Nt, int Ns, int R, const __nv_bfloat16* __restrict__ prm,
                                                    const double* __restrict__ dF, float* __restrict__ grad) {
  extern __shared__ __align__(16) unsigned char smem[];
  CnnW& w = *reinterpret_cast<CnnW*>(smem);
  const int Sp = pad_stride(Ns);
  float* a1 = reinterpret_cast<float*>(smem + align16(sizeof(CnnW)));            // rows r0-2 .. r0+R+1
  float* dz2 = a1 + align16((size_t)(R + 4) * CH * Sp * sizeof(float)) / sizeof(float);  // rows r0-1 .. r0+R
  float* dz1 = dz2 + align16((size_t)(R + 2) * CH * Sp * sizeof(float)) / sizeof(float);  // rows r0 .. r0+R-1
  uint8_t* x = reinterpret_cast<uint8_t*>(dz1 + align16((size_t)R * CH * Sp * sizeof(float)) / sizeof(float));
  float* acc = reinterpret_cast<float*>(x + align16((size_t)(R + 6) * Ns));     // 64 floats: S2 (g a2), db2, db1
  load_cnn_weights(w, prm);
  const int tid = threadIdx.x;
  if (tid < 64) acc[tid] = 0.0f;
  const int o2 = tid >> 4, c2 = tid & 15;              // dW2 owner (blockDim == 256)
  const int o1 = tid / 9, tap1 = tid % 9;              // dW1 owner (tid < 144)
  float gw2[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float gw1[4] = {0, 0, 0, 0};
  float s2[CH], gb2[CH];
#pragma unroll
  for (int o = 0; o < CH; ++o) s2[o] = gb2[o] = 0.0f;
  float gb1 = 0.0f;
  const int tiles = (Nt + R - 1) / R;
  for (int item = blockIdx.x; item < tiles * B; item += gridDim.x) {
    const int b = item / tiles, r0 = (item - b * tiles) * R;
    const uint8_t* s = fields + (size_t)(idx ? idx[b] : b) * Nt * Ns;
    const float g = (float)dF[b];
    __syncthreads();   // the previous item's buffers are no longer read
    for (int e = tid; e < (R + 6) * Ns; e += blockDim.x) {
      const int rr = e / Ns, j = e - rr * Ns;
      x[e] = s[(size_t)wrapi(r0 - 3 + rr, Nt) * Ns + j];
    }
    __syncthreads();
    for (int e = tid; e < (R + 4) * CH * Ns; e += blockDim.x) {
      const int j = e % Ns, o = (e / Ns) % CH, rr = e / (Ns * CH);
      a1[(rr * CH + o) * Sp + j] = cnn_a1(w, o, [&](int dt, int dj) { return (int)x[(rr + 1 + dt) * Ns + wrap1(j + dj, Ns)]; });
    }
    __syncthreads();
    for (int p = tid; p < (R + 2) * Ns; p += blockDim.x) {
      const int rr = p / Ns, j = p - rr * Ns;          // t = r0 - 1 + rr
      const bool own = rr >= 1 && rr <= R && r0 + rr - 1 < Nt;
      float z[CH];
      cnn_z2(w, z, [&](int c, int dt, int dj) { return a1[((rr + 1 + dt) * CH + c) * Sp + wrap1(j + dj, Ns)]; });
#pragma unroll
      for (int o = 0; o < CH; ++o) {
        const float a = tanhf(z[o]);
        const float d = g * w.w3s[o] * (1.0f - a * a);
        dz2[(rr * CH + o) * Sp + j] = d;
        if (own) {
          s2[o] = fmaf(g, a, s2[o]);
          gb2[o] += d;
        }
      }
    }
    __syncthreads();
    // dW2[o][c][tap] += sum over the tile's positions of dz2[o] a1[c] (shifted)
    for (int rr = 0; rr < R && r0 + rr < Nt; ++rr)
      for (int j = 0; j < Ns; ++j) {
        const float d = dz2[((rr + 1) * CH + o2) * Sp + j];
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
          const int dy = tap / 3, dx = tap % 3;
          gw2[tap] = fmaf(d, a1[((rr + 1 + dy) * CH + c2) * Sp + wrap1(j + dx - 1, Ns)], gw2[tap]);
        }
      }
    // da1 at the tile's positions, then dz1 = da1 (1 - a1^2)
    for (int p = tid; p < R * Ns; p += blockDim.x) {
      const int rr = p / Ns, j = p - rr * Ns;
      if (r0 + rr >= Nt) continue;
      float da[CH];
#pragma unroll
      for (int c = 0; c < CH; ++c) da[c] = 0.0f;
      for (int o = 0; o < CH; ++o)
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
          const int dy = tap / 3, dx = tap % 3;
          const float v = dz2[((rr + 2 - dy) * CH + o) * Sp + wrap1(j + 1 - dx, Ns)];
          const float4* wv = reinterpret_cast<const float4*>(&w.w2b[(o * 9 + tap) * 16]);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const float4 ww = wv[q];
            da[4 * q + 0] = fmaf(ww.x, v, da[4 * q + 0]);
            da[4 * q + 1] = fmaf(ww.y, v, da[4 * q + 1]);
            da[4 * q + 2] = fmaf(ww.z, v, da[4 * q + 2]);
            da[4 * q + 3] = fmaf(ww.w, v, da[4 * q + 3]);
          }
        }
#pragma unroll
      for (int c = 0; c < CH; ++c) {
        const float a = a1[((rr + 2) * CH + c) * Sp + j];
        dz1[(rr * CH + c) * Sp + j] = da[c] * (1.0f - a * a);
      }
    }
    __syncthreads();
    // dW1[o][c][tap] += sum of dz1[o] where the shifted field equals c + 1; db1
    if (tid < 144) {
      const int dy = tap1 / 3, dx = tap1 % 3;
      for (int rr = 0; rr < R && r0 + rr < Nt; ++rr)
        for (int j = 0; j < Ns; ++j) {
          const float d = dz1[(rr * CH + o1) * Sp + j];
          const int v = x[(rr + 2 + dy) * Ns + wrap1(j + dx - 1, Ns)] - 1;
          gw1[0] += v == 0 ? d : 0.0f;
          gw1[1] += v == 1 ? d : 0.0f;
          gw1[2] += v == 2 ? d : 0.0f;
          gw1[3] += v == 3 ? d : 0.0f;
        }
    } else if (tid < 160) {
      const int o = tid - 144;
      for (int rr = 0; rr < R && r0 + rr < Nt; ++rr)
        for (int j = 0; j < Ns; ++j) gb1 += dz1[(rr * CH + o) * Sp + j];
    }
  }
  // flush the partials
#pragma unroll
  for (int tap = 0; tap < 9; ++tap) atomicAdd(&grad[KDQ_CNN_OFF_W2 + o2 * 144 + c2 * 9 + tap], gw2[tap]);
  if (tid < 144)
    for (int c = 0; c < 4; ++c) atomicAdd(&grad[KDQ_CNN_OFF_W1 + o1 * 36 + c * 9 + tap1], gw1[c]);
  else if (tid < 160)
    atomicAdd(&grad[KDQ_CNN_OFF_B1 + tid - 144], gb1);
#pragma unroll
  for (int o = 0; o < CH; ++o) {
    atomicAdd(&acc[o], s2[o]);
    atomicAdd(&acc[16 + o], gb2[o]);
  }
  __syncthreads();
  if (tid < CH) {
    for (int tap = 0; tap < 9; ++tap) atomicAdd(&grad[KDQ_CNN_OFF_W3 + tid * 9 + tap], acc[tid]);
    atomicAdd(&grad[KDQ_CNN_OFF_B2 + tid], acc[16 + tid]);
  }
}

// squared-error loss of one batch: dF = 2 (F - y) / B, the b3 gradient
// (F depends on b3 through Nt Ns b3) and the loss sum
__global__ void k_cnn_loss(const double* F, const double* y, const int* idx, int B, int Nt, int Ns, double* dF,
                           float* grad, double* loss) {
  __shared__ double red[2][32];
  double l = 0.0, gs = 0.0;
  for (int b = threadIdx.x; b < B; b += blockDim.x) {
    const double e = F[b] - y[idx ? idx[b] : b];
    dF[b] = 2.0 * e / B;
    l += e * e;
    gs += 2.0 * e / B;
  }
  for (int o = 16; o > 0; o >>= 1) {
    l += __shfl_xor_sync(0xffffffffu, l, o);
    gs += __shfl_xor_sync(0xffffffffu, gs, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = l;
    red[1][threadIdx.x >> 5] = gs;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double L = 0.0, S = 0.0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      L += red[0][q];
      S += red[1][q];
    }
    *loss += L;
    grad[KDQ_CNN_OFF_B3] += (float)(S * Nt * Ns);
  }
}

__global__ void k_cnn_b3_grad(const double* dF, int B, int Nt, int Ns, float* grad) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double S = 0.0;
    for (int b = 0; b < B; ++b) S += dF[b];
    grad[KDQ_CNN_OFF_B3] += (float)(S * Nt * Ns);
  }
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; refreshes the bf16
// copy the kernels compute with and clears the gradient.
__global__ void k_cnn_adam(float* p, float* m, float* v, float* grad, __nv_bfloat16* pb, int n, float lr, float b1,
                           float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float g = grad[i];
    const float mi = b1 * m[i] + (1.0f - b1) * g;
    const float vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / c1, vh = vi / c2;
    const float pi = p[i] - lr * mh / (sqrtf(vh) + eps);
    p[i] = pi;
    pb[i] = __float2bfloat16_rn(pi);
    grad[i] = 0.0f;
  }
}

__global__ void k_to_bf16(const float* p, __nv_bfloat16* pb, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) pb[i] = __float2bfloat16_rn(p[i]);
}

// --------------------------------------------------------------- host side
struct Dev {
  void* p = nullptr;
  ~Dev() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t b) { return cudaMalloc(&p, b ? b : 1); }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

int err(int code, const std::string& m) {
  kdq::set_global_error(m);
  return code;
}

#define CNN_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t _e = (call);                                                             \
    if (_e != cudaSuccess) return err(KDQ_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

int pick_rows(int Ns, int* Rf, int* Rb) {
  *Rf = *Rb = 0;
  for (int R : {4, 2, 1})
    if (!*Rf && fwd_smem(R, Ns) <= SMEM_MAX) *Rf = R;
  for (int R : {4, 2, 1})
    if (!*Rb && bwd_smem(R, Ns) <= SMEM_MAX) *Rb = R;
  return *Rf && *Rb;
}

int check_shape(int n_cfg, int Nt, int Ns) {
  if (n_cfg < 1 || Nt < 1 || Ns < 3 || Ns > 1024) return err(KDQ_ERR_ARG, "kdq_cnn: need n_cfg >= 1, Nt >= 1, 3 <= Ns <= 1024");
  return KDQ_OK;
}

// The kernels of one pass over a batch: forward, (loss), backward.
struct Net {
  int Nt, Ns, Rf, Rb, sms;
  cudaStream_t st = nullptr;
  cudaError_t fwd(const uint8_t* f, const int* idx, int B, const __nv_bfloat16* pb, double* F) {
    cudaError_t e = cudaMemsetAsync(F, 0, B * sizeof(double), st);
    if (e) return e;
    dim3 grid((Nt + Rf - 1) / Rf, B);
    k_cnn_fwd<<<grid, 256, fwd_smem(Rf, Ns), st>>>(f, idx, Nt, Ns, Rf, pb, F);
    return cudaGetLastError();
  }
  cudaError_t bwd(const uint8_t* f, const int* idx, int B, const __nv_bfloat16* pb, const double* dF, float* g) {
    const int items = ((Nt + Rb - 1) / Rb) * B;
    k_cnn_bwd<<<std::min(items, sms), 256, bwd_smem(Rb, Ns), st>>>(f, idx, B, Nt, Ns, Rb, pb, dF, g);
    return cudaGetLastError();
  }
};

// Tile autotuner: the slices per work item (R) of the forward and of the
// backward kernel are timed on the first batch for every R that fits the
// shared memory, and the fastest pair is kept per (Nt, Ns, batch, device).
std::mutex g_tune_mu;
std::map<std::tuple<int, int, int, int>, std::pair<int, int>> g_tuned;

template <class F>
float time_ms(cudaStream_t st, F&& launch) {
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  launch();   // warm-up
  cudaEventRecord(a, st);
  for (int q = 0; q < 3; ++q) launch();
  cudaEventRecord(b, st);
  cudaEventSynchronize(b);
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

int autotune(Net& n, const uint8_t* f, const int* idx, int B, const __nv_bfloat16* pb, double* F, double* dF,
             float* g, int device) {
  const auto key = std::make_tuple(n.Nt, n.Ns, B, device);
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tuned.find(key);
    if (it != g_tuned.end()) {
      n.Rf = it->second.first;
      n.Rb = it->second.second;
      return KDQ_OK;
    }
  }
  const int rf0 = n.Rf, rb0 = n.Rb;   // the largest feasible heights (shared memory opened to these)
  std::vector<double> ones(B, 1.0 / B);
  CNN_CUDA(cudaMemcpy(dF, ones.data(), B * sizeof(double), cudaMemcpyHostToDevice));
  float best_f = 1e30f, best_b = 1e30f;
  int rf = rf0, rb = rb0;
  for (int R : {4, 2, 1}) {
    if (R <= rf0) {
      n.Rf = R;
      const float t = time_ms(n.st, [&] { n.fwd(f, idx, B, pb, F); });
      if (t < best_f) { best_f = t; rf = R; }
    }
    if (R <= rb0) {
      n.Rb = R;
      const float t = time_ms(n.st, [&] { n.bwd(f, idx, B, pb, dF, g); });
      if (t < best_b) { best_b = t; rb = R; }
    }
  }
  CNN_CUDA(cudaGetLastError());
  CNN_CUDA(cudaMemset(g, 0, KDQ_CNN_NPARAM * sizeof(float)));
  n.Rf = rf;
  n.Rb = rb;
  std::lock_guard<std::mutex> lk(g_tune_mu);
  g_tuned[key] = {rf, rb};
  return KDQ_OK;
}

int net_setup(Net& n, int Nt, int Ns, int device) {
  n.Nt = Nt;
  n.Ns = Ns;
  if (!pick_rows(Ns, &n.Rf, &n.Rb)) return err(KDQ_ERR_ARG, "kdq_cnn: lattice too large for the shared-memory tiles");
  CNN_CUDA(cudaSetDevice(device));
  CNN_CUDA(cudaDeviceGetAttribute(&n.sms, cudaDevAttrMultiProcessorCount, device));
  CNN_CUDA(cudaFuncSetAttribute(k_cnn_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fwd_smem(n.Rf, Ns)));
  CNN_CUDA(cudaFuncSetAttribute(k_cnn_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bwd_smem(n.Rb, Ns)));
  return KDQ_OK;
}
}  // namespace

extern "C" int kdq_cnn_forward(const uint8_t* fields, int32_t n_cfg, int32_t Nt, int32_t Ns, const float* params,
                               double* F, int32_t device) {
  if (!fields || !params || !F) return err(KDQ_ERR_ARG, "kdq_cnn_forward: NULL argument");
  if (int rc = check_shape(n_cfg, Nt, Ns)) return rc;
  Net n;
  if (int rc = net_setup(n, Nt, Ns, device)) return rc;
  Dev dfld, dp, dpb, dF;
  const size_t fb = (size_t)n_cfg * Nt * Ns;
  CNN_CUDA(dfld.alloc(fb));
  CNN_CUDA(dp.alloc(KDQ_CNN_NPARAM * sizeof(float)));
  CNN_CUDA(dpb.alloc(KDQ_CNN_NPARAM * sizeof(__nv_bfloat16)));
  CNN_CUDA(dF.alloc(n_cfg * sizeof(double)));
  CNN_CUDA(cudaMemcpy(dfld.p, fields, fb, cudaMemcpyHostToDevice));
  CNN_CUDA(cudaMemcpy(dp.p, params, KDQ_CNN_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  k_to_bf16<<<4, 1024>>>(dp.as<float>(), dpb.as<__nv_bfloat16>(), KDQ_CNN_NPARAM);
  CNN_CUDA(cudaGetLastError());
  CNN_CUDA(n.fwd(dfld.as<uint8_t>(), nullptr, n_cfg, dpb.as<__nv_bfloat16>(), dF.as<double>()));
  CNN_CUDA(cudaMemcpy(F, dF.p, n_cfg * sizeof(double), cudaMemcpyDeviceToHost));
  return KDQ_OK;
}

extern "C" int kdq_cnn_grad(const uint8_t* fields, const double* dF, int32_t n_cfg, int32_t Nt, int32_t Ns,
                            const float* params, float* grad, int32_t device) {
  if (!fields || !params || !dF || !grad) return err(KDQ_ERR_ARG, "kdq_cnn_grad: NULL argument");
  if (int rc = check_shape(n_cfg, Nt, Ns)) return rc;
  Net n;
  if (int rc = net_setup(n, Nt, Ns, device)) return rc;
  Dev dfld, dp, dpb, ddF, dg;
  const size_t fb = (size_t)n_cfg * Nt * Ns;
  CNN_CUDA(dfld.alloc(fb));
  CNN_CUDA(dp.alloc(KDQ_CNN_NPARAM * sizeof(float)));
  CNN_CUDA(dpb.alloc(KDQ_CNN_NPARAM * sizeof(__nv_bfloat16)));
  CNN_CUDA(ddF.alloc(n_cfg * sizeof(double)));
  CNN_CUDA(dg.alloc(KDQ_CNN_NPARAM * sizeof(float)));
  CNN_CUDA(cudaMemcpy(dfld.p, fields, fb, cudaMemcpyHostToDevice));
  CNN_CUDA(cudaMemcpy(dp.p, params, KDQ_CNN_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  CNN_CUDA(cudaMemcpy(ddF.p, dF, n_cfg * sizeof(double), cudaMemcpyHostToDevice));
  CNN_CUDA(cudaMemset(dg.p, 0, KDQ_CNN_NPARAM * sizeof(float)));
  k_to_bf16<<<4, 1024>>>(dp.as<float>(), dpb.as<__nv_bfloat16>(), KDQ_CNN_NPARAM);
  CNN_CUDA(cudaGetLastError());
  CNN_CUDA(n.bwd(dfld.as<uint8_t>(), nullptr, n_cfg, dpb.as<__nv_bfloat16>(), ddF.as<double>(), dg.as<float>()));
  k_cnn_b3_grad<<<1, 32>>>(ddF.as<double>(), n_cfg, Nt, Ns, dg.as<float>());
  CNN_CUDA(cudaGetLastError());
  CNN_CUDA(cudaMemcpy(grad, dg.p, KDQ_CNN_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  return KDQ_OK;
}

extern "C" int kdq_cnn_train(const uint8_t* fields, const double* target, int32_t n_cfg, int32_t Nt, int32_t Ns,
                             int32_t epochs, int32_t batch, float lr, uint64_t seed, float* params,
                             double* loss_per_epoch, int32_t device) {
  if (!fields || !target || !params) return err(KDQ_ERR_ARG, "kdq_cnn_train: NULL argument");
  if (int rc = check_shape(n_cfg, Nt, Ns)) return rc;
  if (epochs < 0 || batch < 1 || !(lr > 0.0f)) return err(KDQ_ERR_ARG, "kdq_cnn_train: need epochs >= 0, batch >= 1, lr > 0");
  Net n;
  if (int rc = net_setup(n, Nt, Ns, device)) return rc;
  batch = std::min(batch, (int)n_cfg);
  const int nb = n_cfg / batch;     // full batches per epoch (the remainder is left out of that epoch)
  Dev dfld, dy, dp, dm, dv, dg, dpb, dF, ddF, didx, dloss;
  const size_t fb = (size_t)n_cfg * Nt * Ns;
  CNN_CUDA(dfld.alloc(fb));
  CNN_CUDA(dy.alloc(n_cfg * sizeof(double)));
  CNN_CUDA(dp.alloc(KDQ_CNN_NPARAM * sizeof(float)));
  CNN_CUDA(dm.alloc(KDQ_CNN_NPARAM * sizeof(float)));
  CNN_CUDA(dv.alloc(KDQ_CNN_NPARAM * sizeof(float)));
  CNN_CUDA(dg.alloc(KDQ_CNN_NPARAM * sizeof(float)));
  CNN_CUDA(dpb.alloc(KDQ_CNN_NPARAM * sizeof(__nv_bfloat16)));
  CNN_CUDA(dF.alloc(batch * sizeof(double)));
  CNN_CUDA(ddF.alloc(batch * sizeof(double)));
  CNN_CUDA(didx.alloc((size_t)n_cfg * sizeof(int)));
  CNN_CUDA(dloss.alloc(std::max(epochs, 1) * sizeof(double)));
  CNN_CUDA(cudaMemcpy(dfld.p, fields, fb, cudaMemcpyHostToDevice));
  CNN_CUDA(cudaMemcpy(dy.p, target, n_cfg * sizeof(double), cudaMemcpyHostToDevice));
  CNN_CUDA(cudaMemcpy(dp.p, params, KDQ_CNN_NPARAM * sizeof(float), cudaMemcpyHostToDevice));
  CNN_CUDA(cudaMemset(dm.p, 0, KDQ_CNN_NPARAM * sizeof(float)));
  CNN_CUDA(cudaMemset(dv.p, 0, KDQ_CNN_NPARAM * sizeof(float)));
  CNN_CUDA(cudaMemset(dg.p, 0, KDQ_CNN_NPARAM * sizeof(float)));
  CNN_CUDA(cudaMemset(dloss.p, 0, std::max(epochs, 1) * sizeof(double)));
  k_to_bf16<<<4, 1024>>>(dp.as<float>(), dpb.as<__nv_bfloat16>(), KDQ_CNN_NPARAM);
  CNN_CUDA(cudaGetLastError());
  if (int rc = autotune(n, dfld.as<uint8_t>(), nullptr, batch, dpb.as<__nv_bfloat16>(), dF.as<double>(),
                        ddF.as<double>(), dg.as<float>(), device))
    return rc;
  std::vector<int> perm(n_cfg);
  std::iota(perm.begin(), perm.end(), 0);
  std::mt19937_64 rng(seed);
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  long long step = 0;
  for (int ep = 0; ep < epochs; ++ep) {
    for (int i = n_cfg - 1; i > 0; --i) std::swap(perm[i], perm[(size_t)(rng() % (uint64_t)(i + 1))]);
    CNN_CUDA(cudaMemcpy(didx.p, perm.data(), (size_t)n_cfg * sizeof(int), cudaMemcpyHostToDevice));
    for (int q = 0; q < nb; ++q) {
      const int* ix = didx.as<int>() + (size_t)q * batch;
      CNN_CUDA(n.fwd(dfld.as<uint8_t>(), ix, batch, dpb.as<__nv_bfloat16>(), dF.as<double>()));
      k_cnn_loss<<<1, 256>>>(dF.as<double>(), dy.as<double>(), ix, batch, Nt, Ns, ddF.as<double>(), dg.as<float>(),
                             dloss.as<double>() + ep);
      CNN_CUDA(cudaGetLastError());
      CNN_CUDA(n.bwd(dfld.as<uint8_t>(), ix, batch, dpb.as<__nv_bfloat16>(), ddF.as<double>(), dg.as<float>()));
      ++step;
      const float c1 = 1.0f - std::pow(b1, (float)step), c2 = 1.0f - std::pow(b2, (float)step);
      k_cnn_adam<<<4, 1024>>>(dp.as<float>(), dm.as<float>(), dv.as<float>(), dg.as<float>(),
                              dpb.as<__nv_bfloat16>(), KDQ_CNN_NPARAM, lr, b1, b2, eps, c1, c2);
      CNN_CUDA(cudaGetLastError());
    }
  }
  CNN_CUDA(cudaDeviceSynchronize());
  CNN_CUDA(cudaMemcpy(params, dp.p, KDQ_CNN_NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
  if (loss_per_epoch && epochs > 0) {
    std::vector<double> l(epochs);
    CNN_CUDA(cudaMemcpy(l.data(), dloss.p, epochs * sizeof(double), cudaMemcpyDeviceToHost));
    for (int ep = 0; ep < epochs; ++ep) loss_per_epoch[ep] = l[ep] / std::max(1, nb * batch);
  }
  return KDQ_OK;
}
