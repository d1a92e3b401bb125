// Effective model of self-learning Monte Carlo: a periodic three-layer
// convolutional net over the slice x site Hubbard-Stratonovich field.
//
//   x[c][t][j]  = [s(t, j) == c + 1]                      (one-hot, 4 channels)
//   a1[o][t][j] = tanh(b1[o] + sum_{c,dy,dx} W1[o][c][dy][dx] x[c][t+dy-1][j+dx-1])
//   a2[o][t][j] = tanh(b2[o] + sum_{c,dy,dx} W2[o][c][dy][dx] a1[c][t+dy-1][j+dx-1])
//   y[t][j]     = b3 + sum_{c,dy,dx} W3[c][dy][dx] a2[c][t+dy-1][j+dx-1]
//   F(s)        = sum_{t,j} y[t][j]
//
// with 16 channels, 3x3 kernels and periodic boundaries in both the slice
// (t mod Nt) and the site index (j mod Ns) directions.  F approximates the
// fermion part 2 log|det(P^H B(Theta,0) P)| of the t-U log-weight.  Because
// the last layer is linear and the sum runs over a periodic domain,
// F = Nt Ns b3 + sum_{c,t,j} w3s[c] a2[c][t][j] with w3s[c] = sum_{dy,dx} W3[c][dy][dx]:
// the kernels use this exact identity, so layer 3 needs no halo.
//
// Parameters are kept as an FP32 master vector (KDQ_CNN_NPARAM floats in
// the order W1, b1, W2, b2, W3, b3, each row-major over the indices above);
// every product uses the bf16-rounded weights with FP32 accumulation.
#pragma once
#include <cuda_bf16.h>
#include <cstdint>

#define KDQ_CNN_CH 16
#define KDQ_CNN_OFF_W1 0
#define KDQ_CNN_OFF_B1 576
#define KDQ_CNN_OFF_W2 592
#define KDQ_CNN_OFF_B2 2896
#define KDQ_CNN_OFF_W3 2912
#define KDQ_CNN_OFF_B3 3056
#define KDQ_CNN_NPARAM 3057

namespace kdq {

// Weights staged in shared memory as FP32 (values of the bf16 weights), in
// the layouts the inner loops read as float4 vectors.
struct __align__(16) CnnW {
  float w1[KDQ_CNN_CH * 4 * 9];          // [o][c][tap]
  float b1[KDQ_CNN_CH];
  float w2f[KDQ_CNN_CH * 9 * KDQ_CNN_CH];  // [c][tap][o]   (forward: 16 outputs per input)
  float w2b[KDQ_CNN_CH * 9 * KDQ_CNN_CH];  // [o][tap][c]   (backward: 16 inputs per output)
  float b2[KDQ_CNN_CH];
  float w3s[KDQ_CNN_CH];                 // sum over taps of W3[c]
  float b3;
};

// Shared-memory bytes of the sweep's cluster moves for clusters of Lc sites:
// the weights, the layer-1 window (7 rows x Lc+6 sites x 16 channels), the
// layer-2 window (5 x Lc+4 x 16), the trial activations of the 3x3 and 5x5
// neighbourhoods of a site and three index arrays of 32.
__host__ __device__ inline size_t slmc_smem_bytes(int Lc) {
  const size_t w = (sizeof(CnnW) + 15) & ~size_t(15);
  return w + sizeof(float) * (7 * 16 * (size_t)(Lc + 6) + 5 * 16 * (size_t)(Lc + 4) + 144 + 400) + 3 * 32 * sizeof(int);
}

__device__ inline void load_cnn_weights(CnnW& w, const __nv_bfloat16* p) {
  for (int e = threadIdx.x; e < KDQ_CNN_CH * 36; e += blockDim.x) w.w1[e] = __bfloat162float(p[KDQ_CNN_OFF_W1 + e]);
  for (int e = threadIdx.x; e < KDQ_CNN_CH * 144; e += blockDim.x) {
    const int o = e / 144, c = (e / 9) % 16, tap = e % 9;
    const float v = __bfloat162float(p[KDQ_CNN_OFF_W2 + e]);
    w.w2f[(c * 9 + tap) * 16 + o] = v;
    w.w2b[(o * 9 + tap) * 16 + c] = v;
  }
  if (threadIdx.x < KDQ_CNN_CH) {
    const int o = threadIdx.x;
    w.b1[o] = __bfloat162float(p[KDQ_CNN_OFF_B1 + o]);
    w.b2[o] = __bfloat162float(p[KDQ_CNN_OFF_B2 + o]);
    float s = 0.0f;
    for (int tap = 0; tap < 9; ++tap) s += __bfloat162float(p[KDQ_CNN_OFF_W3 + o * 9 + tap]);
    w.w3s[o] = s;
  }
  if (threadIdx.x == 0) w.b3 = __bfloat162float(p[KDQ_CNN_OFF_B3]);
  __syncthreads();
}

__device__ __forceinline__ int wrapi(int v, int n) {
  v %= n;
  return v < 0 ? v + n : v;
}

// Layer-1 activation at one position from a field window: `xs(dt, dj)`
// returns the field value (1..4) at offset (dt, dj) in {-1,0,1}^2.
template <class XS>
__device__ __forceinline__ float cnn_a1(const CnnW& w, int o, XS xs) {
  float acc = w.b1[o];
#pragma unroll
  for (int dy = 0; dy < 3; ++dy)
#pragma unroll
    for (int dx = 0; dx < 3; ++dx) acc += w.w1[o * 36 + (xs(dy - 1, dx - 1) - 1) * 9 + dy * 3 + dx];
  return tanhf(acc);
}

// Layer-2 pre-activations (16 outputs) at one position: `a1(c, dt, dj)`
// returns the layer-1 activation of channel c at offset (dt, dj).
template <class A1>
__device__ __forceinline__ void cnn_z2(const CnnW& w, float (&z)[KDQ_CNN_CH], A1 a1) {
#pragma unroll
  for (int o = 0; o < KDQ_CNN_CH; ++o) z[o] = w.b2[o];
  for (int c = 0; c < KDQ_CNN_CH; ++c)
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
      const float v = a1(c, tap / 3 - 1, tap % 3 - 1);
      const float4* wv = reinterpret_cast<const float4*>(&w.w2f[(c * 9 + tap) * 16]);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float4 ww = wv[q];
        z[4 * q + 0] = fmaf(ww.x, v, z[4 * q + 0]);
        z[4 * q + 1] = fmaf(ww.y, v, z[4 * q + 1]);
        z[4 * q + 2] = fmaf(ww.z, v, z[4 * q + 2]);
        z[4 * q + 3] = fmaf(ww.w, v, z[4 * q + 3]);
      }
    }
}

}  // namespace kdq
