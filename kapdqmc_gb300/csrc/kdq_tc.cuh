// Split-precision (3xTF32) products of the mixed-precision sweep on the
// tensor pipe: complex FP32 matrices times the real FP32 kinetic matrices
// (eK, eKinv, HalfeK, HalfeKinv of a hopping matrix without flux;
// tc_cgemm), and complex times complex (tc_zgemm: the two products that
// form G at a recompute, and the delayed rank-k flushes of G).
//
// Every FP32 operand x is split into two TF32 values, hi = tf32(x) and
// lo = tf32(x - hi) (x - hi is exact in FP32), and each product A B is
// accumulated in FP32 as A_lo B_hi + A_hi B_lo + A_hi B_hi (the A_lo B_lo
// term, ~2^-22 relative, is dropped): about FP32 accuracy from TF32 tensor
// operations.  Tiles are mma.sync.m16n8k8 (TF32 inputs, FP32 accumulators);
// the whole CTA computes one product, each warp a 3 x 4 block of 16 x 8
// tiles, operands read through L1.  The kinetic matrices, constant and
// shared by every chain, are split once into fragment order (kin_frag) and
// stay in L2; the other operands are split as they are loaded.
//
// A complex matrix is used through a real view of its interleaved (re, im)
// floats, arranged so that the real and imaginary part of one complex entry
// land in the same thread's accumulators:
//   left  C = A_real B_cplx: real view of B and C has 2N columns, column
//         2j + r = part r of complex column j (an 8-column tile = 4 complex
//         columns; accumulators c0/c1 are re/im of one entry);
//   right C = A_cplx B_real: real view of A and C has 2M rows, tile rows
//         0..7 = re and 8..15 = im of 8 complex rows (c0/c2 and c1/c3).
// The epilogue applies the optional complex row and column scalings
// C = rs[i] (A B)[i,j] cs[j] of the slice wraps and block products.
//
// Reference products (KAPDQMC): WrapKV! src/tU/GreenMatrix.jl:56-86 (and
// src/tUV/GreenMatrix.jl:92-122), BM_F! src/tU/GreenMatrix.jl:10-27, the
// measurement wraps of phy_measure src/tU/phy_update.jl:154-182, the
// products of get_G! src/public/Gupdate.jl:139-157 and the G update of
// Gupdate! src/public/Gupdate.jl:5-11 (applied in batches).
#pragma once
#include <cstdint>

#include "kdq_device.cuh"

namespace kdq {

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void tf32_split(float x, uint32_t& hi, uint32_t& lo) {
  hi = tf32_rna(x);
  lo = tf32_rna(__fsub_rn(x, __uint_as_float(hi)));
}

// d += a b for one m16n8k8 TF32 tile (FP32 accumulators)
__device__ __forceinline__ void mma_tf32(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1) {
  asm(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

constexpr int TC_WM = 3;   // m16 tiles per warp
constexpr int TC_WN = 4;   // n8 tiles per warp

// Pre-split kinetic matrices.  A real N x N kinetic matrix (column-major) is
// constant over the sweep and shared by every chain, so its TF32 hi/lo split
// is done once, into the order in which a warp's lanes consume it:
//   left operand (A of kin X): m16 x k8 tile (mt, kt) of ceil(N/16) x
//     ceil(N/8), lane (g, t): uint4 words 2 w and 2 w + 1 with
//     w = (mt ceil(N/8) + kt) 32 + lane hold hi and lo of a0..a3 =
//     A(16 mt + g, 8 kt + t), A(+8, 8 kt + t), A(16 mt + g, 8 kt + t + 4),
//     A(+8, 8 kt + t + 4);
//   right operand (B of X kin): k8 x n8 tile (kt, nt) of ceil(N/8) x
//     ceil(N/8), lane (g, t): word (kt ceil(N/8) + nt) 32 + lane =
//     (hi b0, hi b1, lo b0, lo b1), b0 = B(8 kt + t, 8 nt + g),
//     b1 = B(8 kt + t + 4, 8 nt + g);
// entries outside the matrix are 0.  The split is the one tc_cgemm applies
// on the fly, so the products are bit for bit the same.
__host__ __device__ inline size_t kin_frag_words(int N) {
  const size_t m16 = (N + 15) / 16, k8 = (N + 7) / 8;
  const size_t left = m16 * k8 * 64, right = k8 * k8 * 32;
  return left > right ? left : right;
}

// C (M x N complex) = rs .* (kin X) .* cs when LEFT (M = K = the kinetic
// matrix's order), rs .* (X kin) .* cs otherwise (K = N = its order), with
// the real kinetic matrix kin given by its pre-split words kf (left layout
// for LEFT, right layout otherwise) and X complex (K x N or M x K, ldx
// complex elements).  C must not alias X.  rs (M) and cs (N) may be NULL.
// All threads of the CTA call it; it ends with __syncthreads().
template <bool LEFT>
__device__ __noinline__ void tc_cgemm(int M, int N, int K, const uint4* __restrict__ kf,
                                      const float* __restrict__ X, int ldx, cf* __restrict__ C, int ldc,
                                      const cf* rs, const cf* cs) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  // real-view extents in m16 / n8 tiles
  const int MT = LEFT ? (M + 15) / 16 : (M + 7) / 8;
  const int NT = LEFT ? (N + 3) / 4 : (N + 7) / 8;
  const int KT = (K + 7) / 8;
  const int WMT = (MT + TC_WM - 1) / TC_WM, WNT = (NT + TC_WN - 1) / TC_WN;
  float* Cf = reinterpret_cast<float*>(C);
  for (int wt = warp; wt < WMT * WNT; wt += nwarps) {
    const int mt0 = (wt % WMT) * TC_WM, nt0 = (wt / WMT) * TC_WN;
    float acc[TC_WM][TC_WN][4];
#pragma unroll
    for (int i = 0; i < TC_WM; ++i)
#pragma unroll
      for (int j = 0; j < TC_WN; ++j)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.0f;
    // float offsets of this thread's fragment rows / columns of X (-1: outside)
    int arow[TC_WM][2];   // right: A = X, complex row 8 mt + g, part h (rows g, g + 8 of the tile)
    int bcol[TC_WN];      // left: B = X, complex column 4 nt + g / 2, part g & 1
    if constexpr (!LEFT) {
#pragma unroll
      for (int i = 0; i < TC_WM; ++i)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int mt = mt0 + i, m = mt * 8 + g;
          arow[i][h] = (mt < MT && m < M) ? 2 * m + h : -1;
        }
    } else {
#pragma unroll
      for (int j = 0; j < TC_WN; ++j) {
        const int nt = nt0 + j, n = nt * 4 + (g >> 1);
        bcol[j] = (nt < NT && n < N) ? 2 * n * ldx + (g & 1) : -1;
      }
    }
    for (int kt = 0; kt < KT; ++kt) {
      const int k0 = kt * 8 + t, k1 = k0 + 4;
      const bool kin0 = k0 < K, kin1 = k1 < K;
      uint32_t ah[TC_WM][4], al[TC_WM][4];
      if constexpr (LEFT) {   // kinetic A: its lane's pre-split words
#pragma unroll
        for (int i = 0; i < TC_WM; ++i) {
          const int mt = mt0 + i;
          uint4 h = make_uint4(0u, 0u, 0u, 0u), l = h;
          if (mt < MT) {
            const uint4* w = kf + ((size_t)(mt * KT + kt) * 32 + lane) * 2;
            h = w[0];
            l = w[1];
          }
          ah[i][0] = h.x; ah[i][1] = h.y; ah[i][2] = h.z; ah[i][3] = h.w;
          al[i][0] = l.x; al[i][1] = l.y; al[i][2] = l.z; al[i][3] = l.w;
        }
      } else {                // complex A = X, split here
#pragma unroll
        for (int i = 0; i < TC_WM; ++i) {
          float v[4];
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const int r = arow[i][h];
            v[h] = (r >= 0 && kin0) ? X[r + (size_t)k0 * 2 * ldx] : 0.0f;
            v[2 + h] = (r >= 0 && kin1) ? X[r + (size_t)k1 * 2 * ldx] : 0.0f;
          }
          // fragment order: a0 (row g, col t), a1 (row g+8, col t), a2 (row g, col t+4), a3 (row g+8, col t+4)
#pragma unroll
          for (int q = 0; q < 4; ++q) tf32_split(v[q], ah[i][q], al[i][q]);
        }
      }
      uint32_t bh[TC_WN][2], bl[TC_WN][2];
      if constexpr (LEFT) {   // complex B = X, split here
#pragma unroll
        for (int j = 0; j < TC_WN; ++j) {
          const int c = bcol[j];
          const float v0 = (c >= 0 && kin0) ? X[c + 2 * k0] : 0.0f;
          const float v1 = (c >= 0 && kin1) ? X[c + 2 * k1] : 0.0f;
          tf32_split(v0, bh[j][0], bl[j][0]);
          tf32_split(v1, bh[j][1], bl[j][1]);
        }
      } else {                // kinetic B: its lane's pre-split word
#pragma unroll
        for (int j = 0; j < TC_WN; ++j) {
          const int nt = nt0 + j;
          uint4 v = make_uint4(0u, 0u, 0u, 0u);
          if (nt < NT) v = kf[((size_t)kt * NT + nt) * 32 + lane];
          bh[j][0] = v.x; bh[j][1] = v.y; bl[j][0] = v.z; bl[j][1] = v.w;
        }
      }
#pragma unroll
      for (int i = 0; i < TC_WM; ++i)
#pragma unroll
        for (int j = 0; j < TC_WN; ++j) {
          mma_tf32(acc[i][j], al[i][0], al[i][1], al[i][2], al[i][3], bh[j][0], bh[j][1]);
          mma_tf32(acc[i][j], ah[i][0], ah[i][1], ah[i][2], ah[i][3], bl[j][0], bl[j][1]);
          mma_tf32(acc[i][j], ah[i][0], ah[i][1], ah[i][2], ah[i][3], bh[j][0], bh[j][1]);
        }
    }
    // epilogue: complex entries, optional scalings
#pragma unroll
    for (int i = 0; i < TC_WM; ++i)
#pragma unroll
      for (int j = 0; j < TC_WN; ++j) {
        const int mt = mt0 + i, nt = nt0 + j;
        if (mt >= MT || nt >= NT) continue;
        cf e[2];
        int row[2], col[2];
        if (LEFT) {   // entries (16 mt + g, 4 nt + t) and (16 mt + g + 8, 4 nt + t)
          e[0] = cf{acc[i][j][0], acc[i][j][1]};
          e[1] = cf{acc[i][j][2], acc[i][j][3]};
          row[0] = mt * 16 + g;
          row[1] = row[0] + 8;
          col[0] = col[1] = nt * 4 + t;
        } else {      // entries (8 mt + g, 8 nt + 2t) and (8 mt + g, 8 nt + 2t + 1)
          e[0] = cf{acc[i][j][0], acc[i][j][2]};
          e[1] = cf{acc[i][j][1], acc[i][j][3]};
          row[0] = row[1] = mt * 8 + g;
          col[0] = nt * 8 + 2 * t;
          col[1] = col[0] + 1;
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          if (row[q] >= M || col[q] >= N) continue;
          cf v = e[q];
          if (rs) v = rs[row[q]] * v;
          if (cs) v = v * cs[col[q]];
          *reinterpret_cast<float2*>(Cf + 2 * (row[q] + (size_t)col[q] * ldc)) = make_float2(v.x, v.y);
        }
      }
  }
  __syncthreads();
}

// Word e of the pre-split layouts of the N x N kinetic matrix kin: writes the
// left-operand words 2e, 2e + 1 (e < ceil(N/16) ceil(N/8) 32) into left and
// the right-operand word e (e < ceil(N/8)^2 32) into right.
__device__ inline void kin_frag_word(const float* __restrict__ kin, int N, size_t e, uint4* __restrict__ left,
                                     uint4* __restrict__ right) {
  const int K8 = (N + 7) / 8, M16 = (N + 15) / 16;
  const int lane = (int)(e & 31), g = lane >> 2, t = lane & 3;
  const size_t tile = e >> 5;
  auto at = [&](int r, int k) { return (r < N && k < N) ? kin[r + (size_t)k * N] : 0.0f; };
  if (tile < (size_t)M16 * K8) {
    const int mt = (int)(tile / K8), kt = (int)(tile % K8);
    const int r = 16 * mt + g, k = 8 * kt + t;
    const float v[4] = {at(r, k), at(r + 8, k), at(r, k + 4), at(r + 8, k + 4)};
    uint32_t h[4], l[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) tf32_split(v[q], h[q], l[q]);
    left[2 * e] = make_uint4(h[0], h[1], h[2], h[3]);
    left[2 * e + 1] = make_uint4(l[0], l[1], l[2], l[3]);
  }
  if (tile < (size_t)K8 * K8) {
    const int kt = (int)(tile / K8), nt = (int)(tile % K8);
    uint32_t h0, l0, h1, l1;
    tf32_split(at(8 * kt + t, 8 * nt + g), h0, l0);
    tf32_split(at(8 * kt + t + 4, 8 * nt + g), h1, l1);
    right[e] = make_uint4(h0, h1, l0, l1);
  }
}

// One complex entry (re, im) of a cf (S = 2) or cdf (S = 4, hi + lo) array.
template <int S>
__device__ __forceinline__ void tc_ldc(const float* __restrict__ p, float& re, float& im) {
  if constexpr (S == 4) {
    re = __fadd_rn(p[0], p[1]);
    im = __fadd_rn(p[2], p[3]);
  } else {
    re = p[0];
    im = p[1];
  }
}

// C (M x N complex FP32, ldc) = A B with A (M x K) and B (K x N) complex
// matrices whose entries are SA (SB) floats apart: 2 for cf, 4 for cdf
// (re.hi, re.lo, im.hi, im.lo; the FP32 value hi + lo is used).  Real view:
// C' = A' B' with K' = 2K, real k index 2k + p,
//   A'(re row m, 2k + p) = p ? -Ai[m,k] : Ar[m,k]
//   A'(im row m, 2k + p) = p ?  Ar[m,k] : Ai[m,k]
//   B'(2k + p, n)        = p ?  Bi[k,n] : Br[k,n]
// so that the re / im rows of C' are Ar Br - Ai Bi and Ai Br + Ar Bi; tile
// rows 0..7 = re and 8..15 = im of 8 complex rows, as in tc_cgemm<false>.
// Same 3xTF32 split and warp blocking as tc_cgemm.  BROW: B stored by rows,
// entry (k, n) at SB (k ldb + n).  SUB: C <- C - A B (the accumulators start
// from C).  C must not alias A or B.  All threads of the CTA call it; it ends
// with __syncthreads().
template <int SA, int SB, bool BROW = false, bool SUB = false>
__device__ __noinline__ void tc_zgemm(int M, int N, int K, const float* __restrict__ A, int lda,
                                      const float* __restrict__ B, int ldb, cf* __restrict__ C, int ldc) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const int g = lane >> 2, t = lane & 3, p = t & 1;
  const int MT = (M + 7) / 8, NT = (N + 7) / 8, KT = (K + 3) / 4;
  const int WMT = (MT + TC_WM - 1) / TC_WM, WNT = (NT + TC_WN - 1) / TC_WN;
  float* Cf = reinterpret_cast<float*>(C);
  for (int wt = warp; wt < WMT * WNT; wt += nwarps) {
    const int mt0 = (wt % WMT) * TC_WM, nt0 = (wt / WMT) * TC_WN;
    int arow[TC_WM];   // complex row 8 mt + g of each m tile (-1: outside)
#pragma unroll
    for (int i = 0; i < TC_WM; ++i) {
      const int m = (mt0 + i) * 8 + g;
      arow[i] = (mt0 + i < MT && m < M) ? m : -1;
    }
    int bcol[TC_WN];   // complex column 8 nt + g of each n tile (-1: outside)
#pragma unroll
    for (int j = 0; j < TC_WN; ++j) {
      const int n = (nt0 + j) * 8 + g;
      bcol[j] = (nt0 + j < NT && n < N) ? n : -1;
    }
    float acc[TC_WM][TC_WN][4];
#pragma unroll
    for (int i = 0; i < TC_WM; ++i)
#pragma unroll
      for (int j = 0; j < TC_WN; ++j)
#pragma unroll
        for (int q = 0; q < 2; ++q) {   // this thread's entries (8 mt + g, 8 nt + 2t + q), as in the epilogue
          const int n = (nt0 + j) * 8 + 2 * t + q;
          float re = 0.0f, im = 0.0f;
          if (SUB && arow[i] >= 0 && nt0 + j < NT && n < N) {
            const int o = 2 * (arow[i] + n * ldc);   // M, N <= KDQ_MAX_NS
            re = Cf[o];
            im = Cf[o + 1];
          }
          acc[i][j][q] = re;
          acc[i][j][2 + q] = im;
        }
    for (int kt = 0; kt < KT; ++kt) {
      // real k columns t and t + 4 of the tile: complex k0 and k0 + 2, part p
      const int k0 = kt * 4 + (t >> 1), k1 = k0 + 2;
      const bool kin0 = k0 < K, kin1 = k1 < K;
      uint32_t ah[TC_WM][4], al[TC_WM][4];
#pragma unroll
      for (int i = 0; i < TC_WM; ++i) {
        const int m = arow[i];
        float r0 = 0.0f, i0 = 0.0f, r1 = 0.0f, i1 = 0.0f;
        if (m >= 0 && kin0) tc_ldc<SA>(A + (size_t)SA * (m + (size_t)k0 * lda), r0, i0);
        if (m >= 0 && kin1) tc_ldc<SA>(A + (size_t)SA * (m + (size_t)k1 * lda), r1, i1);
        // fragment order: a0 (re row, k col t), a1 (im row, t), a2 (re row, t + 4), a3 (im row, t + 4)
        const float v[4] = {p ? -i0 : r0, p ? r0 : i0, p ? -i1 : r1, p ? r1 : i1};
#pragma unroll
        for (int q = 0; q < 4; ++q) tf32_split(SUB ? -v[q] : v[q], ah[i][q], al[i][q]);
      }
      uint32_t bh[TC_WN][2], bl[TC_WN][2];
#pragma unroll
      for (int j = 0; j < TC_WN; ++j) {
        const int n = bcol[j];
        float r0 = 0.0f, i0 = 0.0f, r1 = 0.0f, i1 = 0.0f;
        if (n >= 0 && kin0)
          tc_ldc<SB>(B + (size_t)SB * (BROW ? (size_t)k0 * ldb + n : k0 + (size_t)n * ldb), r0, i0);
        if (n >= 0 && kin1)
          tc_ldc<SB>(B + (size_t)SB * (BROW ? (size_t)k1 * ldb + n : k1 + (size_t)n * ldb), r1, i1);
        tf32_split(p ? i0 : r0, bh[j][0], bl[j][0]);
        tf32_split(p ? i1 : r1, bh[j][1], bl[j][1]);
      }
#pragma unroll
      for (int i = 0; i < TC_WM; ++i)
#pragma unroll
        for (int j = 0; j < TC_WN; ++j) {
          mma_tf32(acc[i][j], al[i][0], al[i][1], al[i][2], al[i][3], bh[j][0], bh[j][1]);
          mma_tf32(acc[i][j], ah[i][0], ah[i][1], ah[i][2], ah[i][3], bl[j][0], bl[j][1]);
          mma_tf32(acc[i][j], ah[i][0], ah[i][1], ah[i][2], ah[i][3], bh[j][0], bh[j][1]);
        }
    }
    // entries (8 mt + g, 8 nt + 2t) and (8 mt + g, 8 nt + 2t + 1): re in c0 / c1, im in c2 / c3
#pragma unroll
    for (int i = 0; i < TC_WM; ++i)
#pragma unroll
      for (int j = 0; j < TC_WN; ++j) {
        const int m = arow[i];
        if (m < 0 || nt0 + j >= NT) continue;
#pragma unroll
        for (int q = 0; q < 2; ++q) {
          const int n = (nt0 + j) * 8 + 2 * t + q;
          if (n >= N) continue;
          *reinterpret_cast<float2*>(Cf + 2 * (m + n * ldc)) = make_float2(acc[i][j][q], acc[i][j][2 + q]);
        }
      }
  }
  __syncthreads();
}

}  // namespace kdq
