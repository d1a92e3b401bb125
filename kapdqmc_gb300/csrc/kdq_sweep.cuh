// Sweep kernels: one CTA per Markov chain, one launch per stabilisation
// block.  A launch runs the block's time slices (wrap, local updates,
// optional measurement) and then the QR-stabilised recompute of G at the
// block's closing node, so a full sweep is 2*(NN-1) launches of the same
// kernel (NN = number of nodes).
//
// Two precisions.  T / KT are the FP64 types of the sweep (complex128 or
// float64 for G, float64 or complex128 for the kinetic matrices); TW / KW are
// the working types of the bulk products (slice wraps, thin B-products,
// measurement products) and of the rank-k updates; TS (Ctx::TS) is the type
// of the stabilisation (thin QR, inverse, G recompute).  Plain mode:
// TW = TS = T.  Mixed mode: TW = FP32 (float / complex float), the products
// with a real kinetic matrix on the tensor pipe as 3xTF32 (kdq_tc.cuh), the
// updates delayed; TS = double-float (df / cdf, kdq_device.cuh) on the FP32
// pipe; the acceptance ratios stay FP64 (T).
//
// Reference (KAPDQMC): src/tU/phy_update.jl:3-267, src/tU/GreenMatrix.jl,
// src/tV/phy_update.jl:1-314, src/tV/GreenMatrix.jl,
// src/tUV/phy_update.jl:1-355, src/tUV/GreenMatrix.jl, src/public/Gupdate.jl.
#pragma once
#include <type_traits>

#include "kdq_cnn.cuh"
#include "kdq_device.cuh"
#include "kdq_params.h"
#include "kdq_tc.cuh"

namespace kdq {

constexpr uint32_t PH_M0 = 0xD2511F53u, PH_M1 = 0xCD9E8D57u;
constexpr uint32_t PH_W0 = 0x9E3779B9u, PH_W1 = 0xBB67AE85u;
constexpr uint32_t TAPE_STREAM = 0x4B445131u;

// Philox4x32-10 (Salmon et al., SC'11).
__device__ inline uint4 philox(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) { k0 += PH_W0; k1 += PH_W1; }
    const uint32_t hi0 = __umulhi(PH_M0, c.x), lo0 = PH_M0 * c.x;
    const uint32_t hi1 = __umulhi(PH_M1, c.z), lo1 = PH_M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
  }
  return c;
}

// Register tiles of the block GEMMs per lattice-size class (MAXRM = row
// groups of 32: N <= 32, <= 96, <= 192) and arithmetic: square N x N
// products and thin N x ns / ns x N products.  Chosen so that the tile grid
// fills whole warps at the configured lattice sizes (72 real: 24 x 8 tiles
// of 3 x 9; 64 complex: 32 x 8 tiles of 2 x 8).
template <int MAXRM, class T> struct Tiles;
template <class T> struct Tiles<1, T> { static constexpr int SM = 1, SN = 4, TM = 1, TN = 4; };
template <> struct Tiles<3, double> { static constexpr int SM = 3, SN = 9, TM = 3, TN = 4; };
template <> struct Tiles<3, cd> { static constexpr int SM = 2, SN = 8, TM = 2, TN = 4; };
template <class T> struct Tiles<6, T> { static constexpr int SM = 3, SN = 6, TM = 3, TN = 6; };
template <> struct Tiles<6, cd> { static constexpr int SM = 2, SN = 6, TM = 2, TN = 6; };
template <> struct Tiles<3, float> { static constexpr int SM = 3, SN = 9, TM = 3, TN = 4; };
template <> struct Tiles<3, cf> { static constexpr int SM = 2, SN = 8, TM = 2, TN = 4; };
template <> struct Tiles<3, df> : Tiles<3, double> {};
template <> struct Tiles<3, cdf> : Tiles<3, cd> {};
template <> struct Tiles<6, cdf> : Tiles<6, cd> {};

template <int MAXRM, class T, class TA, class TB, class TC, class TS = double>
__device__ inline void gemm_sq(int M, int N, int K, const TA* A, int lda, const TB* B, int ldb, TC* C,
                               int ldc, const TS* rs = nullptr, const TS* cs = nullptr) {
  bgemm_t<Tiles<MAXRM, T>::SM, Tiles<MAXRM, T>::SN>(M, N, K, A, lda, B, ldb, C, ldc, rs, cs);
}
template <int MAXRM, class T, class TA, class TB, class TC, class TS = double>
__device__ inline void gemm_thin(int M, int N, int K, const TA* A, int lda, const TB* B, int ldb, TC* C,
                                 int ldc, const TS* rs = nullptr, const TS* cs = nullptr) {
  bgemm_t<Tiles<MAXRM, T>::TM, Tiles<MAXRM, T>::TN>(M, N, K, A, lda, B, ldb, C, ldc, rs, cs);
}

// Products with a kinetic matrix kin (eK, eKinv, HalfeK, HalfeKinv):
// C = rs .* (kin X) .* cs (kmul_left) or rs .* (X kin) .* cs (kmul_right).
// The mixed sweep with a real kinetic matrix (no flux) runs them as 3xTF32
// tensor tiles (kdq_tc.cuh) with the kinetic operand pre-split (kf, see
// kin_frag); the FP64 sweep and complex kinetic matrices use the
// register-tiled CUDA-core GEMM (THIN: the N x ns / ns x N tile shape).
enum { KIN_EK = 0, KIN_EKINV = 1, KIN_HALFEK = 2, KIN_HALFEKINV = 3 };

// Pre-split words of kinetic matrix kid as the left (side 0) or right
// (side 1) operand, or NULL (then the TF32 products are not used: the
// runtime builds the words whenever the mixed sweep has a real kinetic
// matrix, and refuses to launch it without them).
__device__ __forceinline__ const uint4* kin_frag(const SweepParams& P, int kid, int side) {
  return P.kin_frag ? static_cast<const uint4*>(P.kin_frag) + (size_t)(2 * kid + side) * P.kin_frag_words
                    : nullptr;
}

template <int MAXRM, bool THIN, class TW, class KW>
__device__ inline void kmul_left(int M, int N, int K, const KW* kin, const uint4* kf, int ldk, const TW* X, int ldx,
                                 TW* C, int ldc, const TW* rs = nullptr, const TW* cs = nullptr) {
  if constexpr (std::is_same_v<TW, cf> && std::is_same_v<KW, float>) {
    tc_cgemm<true>(M, N, K, kf, reinterpret_cast<const float*>(X), ldx, C, ldc, rs, cs);
  } else if constexpr (THIN) {
    gemm_thin<MAXRM, TW>(M, N, K, kin, ldk, X, ldx, C, ldc, rs, cs);
  } else {
    gemm_sq<MAXRM, TW>(M, N, K, kin, ldk, X, ldx, C, ldc, rs, cs);
  }
}
template <int MAXRM, bool THIN, class TW, class KW>
__device__ inline void kmul_right(int M, int N, int K, const TW* X, int ldx, const KW* kin, const uint4* kf, int ldk,
                                  TW* C, int ldc, const TW* rs = nullptr, const TW* cs = nullptr) {
  if constexpr (std::is_same_v<TW, cf> && std::is_same_v<KW, float>) {
    tc_cgemm<false>(M, N, K, kf, reinterpret_cast<const float*>(X), ldx, C, ldc, rs, cs);
  } else if constexpr (THIN) {
    gemm_thin<MAXRM, TW>(M, N, K, X, ldx, kin, ldk, C, ldc, rs, cs);
  } else {
    gemm_sq<MAXRM, TW>(M, N, K, X, ldx, kin, ldk, C, ldc, rs, cs);
  }
}

// ------------------------------------------------------------ phase timing
// Optional per-chain clock counts of the sweep's phases (thread 0, between
// barriers): 0 wraps, 1 local updates (the FP64 sweep's windows of
// acceptance ratios and G updates; the mixed sweep's new update vectors and
// flushes of the delayed updates), 2 measurements, 3 block products of the
// stabilisation chain, 4 QR, 5 G recompute, 6 cluster moves, 7 the mixed
// sweep's windows of acceptance ratios.
struct PhaseClock {
  unsigned long long* acc;
  long long t;
  __device__ void start(unsigned long long* a) {
    acc = a;
    t = a ? clock64() : 0;
  }
  __device__ void lap(int phase) {
    if (!acc) return;
    __syncthreads();
    if (threadIdx.x == 0) {
      const long long now = clock64();
      acc[phase] += (unsigned long long)(now - t);
      t = now;
    }
  }
};

// Per-CTA shared scratch (static part; the tape slice is dynamic); T is the
// working type.
template <class T>
struct Smem {
  double red[32];
  double wn[KDQ_MAX_NS / 2];
  T dvec[KDQ_MAX_NS];   // row scaling of the current slice
  T dinv[KDQ_MAX_NS];   // column scaling
  T ucol[4][KDQ_MAX_NS];   // update vectors: [2 buf + r], two buffers of rank 2
  T wrow[4][KDQ_MAX_NS];
  T rr[4];
  int site[2];     // the accepted proposal's sites (delayed updates)
  int accept[2];
  int nxt[2];      // next proposal of a layer after a window (FP64)
  int newv;
  int bad;
  int nacc;                     // acceptances of the current slice (thread 0)
  uint8_t fld[KDQ_MAX_FIELD];   // the current slice's fields while its proposals run
};

template <int KIND, class T, class KT, class TW, class KW>
struct Ctx {
  // arithmetic of the stabilisation (QR, inverse, G recompute): T in the
  // plain sweep, its double-float counterpart in the mixed one
  using TS = std::conditional_t<std::is_same_v<T, TW>, T, typename dfl_t<T>::type>;
  const SweepParams& P;
  Smem<TW>& sm;
  uint8_t* tk;     // tape slice: choice index
  double* tu;      // tape slice: uniform
  int chain;
  ChainCtl* ctl;
  TW* G;           // equal-time Green's function, working precision
  TW* W1;          // N x N work
  TW* W2;          // N x N work (measurement)
  TW* Yw;          // thin factors in working precision (N x ns)
  TW* Y2w;
  TS* Y;           // thin factors in the stabilisation type (alias Yw, Y2w in plain mode)
  TS* Y2;
  TS* Gd;          // N x N recompute product (alias W1 in plain mode)
  TS* Mss;         // ns x ns (the cluster moves borrow it as T)
  TS* X;
  int* piv;
  uint8_t* s;      // this chain's field, Nt x n_field
  const KW* eK;    // kinetic matrices in working precision
  const KW* eKinv;
  const KW* HalfeK;
  const KW* HalfeKinv;
  const KT* Kmat;  // hopping matrix (observables, FP64)
  PhaseClock& clk;
  unsigned char* slmc = nullptr;   // cluster-move shared memory (dynamic), or NULL
};

// Walks the elements e = tid, tid + nthreads, ... of a column-major M x N
// matrix keeping (row, col) up to date without a division per element.
struct Walk {
  int e, i, j, di, dj, M, total, st;
  __device__ Walk(int M_, int N_) : Walk(M_, N_, threadIdx.x, blockDim.x) {}
  // elements e = start, start + stride, ...
  __device__ Walk(int M_, int N_, int start, int stride) : M(M_), total(M_ * N_), st(stride) {
    e = start;
    i = e % M;
    j = e / M;
    di = st % M;
    dj = st / M;
  }
  __device__ bool ok() const { return e < total; }
  __device__ void next() {
    e += st;
    i += di;
    j += dj;
    if (i >= M) {
      i -= M;
      ++j;
    }
  }
};

// ---------------------------------------------------------------- tables
// Forward (sign=+1) / backward (sign=-1) diagonal factor of slice lt
// (1-based) into sm.dvec, and its elementwise inverse into sm.dinv.
template <int KIND, class T, class KT, class TW, class KW>
__device__ void slice_diag(Ctx<KIND, T, KT, TW, KW>& c, int lt, int sign, const uint8_t* fields = nullptr) {
  const SweepParams& P = c.P;
  const uint8_t* sl = fields ? fields : c.s + (size_t)(lt - 1) * P.n_field;
  if constexpr (KIND == KDQ_TU) {
    // D = cis(±α η_s), 1 ./ D  (src/tU/phy_update.jl:61-63,123-125)
    const cd* tab = reinterpret_cast<const cd*>(P.dtab) + (size_t)(lt - 1) * 16 + (sign > 0 ? 0 : 8);
    for (int i = threadIdx.x; i < P.Ns; i += blockDim.x) {
      const int v = sl[i] - 1;
      c.sm.dvec[i] = cvt<TW>(tab[v]);
      c.sm.dinv[i] = cvt<TW>(tab[4 + v]);
    }
  } else if constexpr (KIND == KDQ_TUV) {
    // phase per site: Σ η over bonds starting at x + a Σ η over bonds ending
    // at x, accumulated in bond order (src/tUV/phy_update.jl:68-78)
    for (int x = threadIdx.x; x < P.Ns; x += blockDim.x) {
      double th = 0.0;
      const int* lst = P.site_bonds + (size_t)x * P.site_nb;
      for (int m = 0; m < P.site_nb; ++m) {
        const int e = lst[m];
        if (e < 0) break;
        const double ev = P.eta[sl[e >> 1] - 1];
        th += (e & 1) ? P.a * ev : ev;
      }
      T d, di;
      if constexpr (sizeof(T) == sizeof(cd)) {
        double sn, cs;
        sincos(sign * th, &sn, &cs);
        cd dd{cs, sn};
        d = dd;
        di = cd{1.0, 0.0} / dd;
      } else {
        const double dd = exp(sign * th);
        d = dd;
        di = 1.0 / dd;
      }
      c.sm.dvec[x] = cvt<TW>(d);
      c.sm.dinv[x] = cvt<TW>(di);
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------------ wraps
// G <- B_lt G B_lt^{-1}, B = D eK (tU, tUV): WrapKV!("Forward","B"),
// src/tU/GreenMatrix.jl:64-69.
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void wrap_fwd_kv(Ctx<KIND, T, KT, TW, KW>& c, TW* G, TW* W, int lt) {
  const int N = c.P.Ns;
  slice_diag(c, lt, +1);
  kmul_left<MAXRM, false>(N, N, N, c.eK, kin_frag(c.P, KIN_EK, 0), N, G, N, W, N);                         // eK G
  kmul_right<MAXRM, false>(N, N, N, W, N, c.eKinv, kin_frag(c.P, KIN_EKINV, 1), N, G, N, c.sm.dvec, c.sm.dinv); // D (.) eKinv D^-1
}

// G <- B_lt^{-1} G B_lt: WrapKV!("Backward","B"), src/tU/GreenMatrix.jl:78-83.
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void wrap_bwd_kv(Ctx<KIND, T, KT, TW, KW>& c, TW* G, TW* W, int lt) {
  const int N = c.P.Ns;
  slice_diag(c, lt, -1);
  for (Walk w(N, N); w.ok(); w.next()) G[w.e] = (c.sm.dvec[w.i] * G[w.e]) * c.sm.dinv[w.j];
  __syncthreads();
  kmul_left<MAXRM, false>(N, N, N, c.eKinv, kin_frag(c.P, KIN_EKINV, 0), N, G, N, W, N);
  kmul_right<MAXRM, false>(N, N, N, W, N, c.eK, kin_frag(c.P, KIN_EK, 1), N, G, N);
}

// tV bond rotation of direction j on both sides of G:
// G <- (UV D UV) G (UV D^-1 UV) (WrapV!(..,"B"), src/tV/GreenMatrix.jl:110-118).
// UV is a direct sum of 2x2 blocks u = [-c -c; -c c] (c = 2^-1/2) over the
// bonds of direction j, a perfect matching, so UV D UV is the direct sum of
// L_b = u diag(d_x, d_y) u = 1/2 [d_x+d_y, d_x-d_y; d_x-d_y, d_x+d_y] and every
// 2x2 block of G (bond b rows, bond b' columns) becomes L_b B R_b'.
// The per-bond coefficients are staged in sm.dvec / sm.dinv as (plus, minus)
// pairs for rows (L) and columns (R).
template <int KIND, class T, class KT, class TW, class KW>
__device__ void tv_coeffs(Ctx<KIND, T, KT, TW, KW>& c, int lt, int j, int sign, const uint8_t* fields = nullptr) {
  const SweepParams& P = c.P;
  const int nb = P.Ns / 2;
  const uint8_t* sl = (fields ? fields : c.s + (size_t)(lt - 1) * P.n_field) + (size_t)j * nb;
  // vtab per slice: [D_x | D_y | 1/D_x | 1/D_y] forward, then the same backward
  const double* tab = P.vtab + (size_t)(lt - 1) * 32 + (sign > 0 ? 0 : 16);
  TW* L = c.sm.dvec;
  TW* R = c.sm.dinv;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    const int v = sl[i] - 1;
    const double dx = tab[v], dy = tab[4 + v], ix = tab[8 + v], iy = tab[12 + v];
    L[2 * i] = cvt<TW>(0.5 * (dx + dy));
    L[2 * i + 1] = cvt<TW>(0.5 * (dx - dy));
    R[2 * i] = cvt<TW>(0.5 * (ix + iy));
    R[2 * i + 1] = cvt<TW>(0.5 * (ix - iy));
  }
  __syncthreads();
}

template <int KIND, class T, class KT, class TW, class KW>
__device__ void tv_rotate(Ctx<KIND, T, KT, TW, KW>& c, TW* G, int lt, int j, int sign) {
  const SweepParams& P = c.P;
  const int N = P.Ns, nb = N / 2;
  tv_coeffs(c, lt, j, sign);
  const TW* L = c.sm.dvec;
  const TW* R = c.sm.dinv;
  const int* bx = P.bx + (size_t)j * nb;
  const int* by = P.by + (size_t)j * nb;
  for (Walk w(nb, nb); w.ok(); w.next()) {
    const int i = w.i, ip = w.j;
    const int x = bx[i], y = by[i], xp = bx[ip], yp = by[ip];
    const TW lp = L[2 * i], lm = L[2 * i + 1], rp = R[2 * ip], rm = R[2 * ip + 1];
    const TW g00 = G[x + (size_t)xp * N], g01 = G[x + (size_t)yp * N];
    const TW g10 = G[y + (size_t)xp * N], g11 = G[y + (size_t)yp * N];
    // L B
    const TW a00 = lp * g00 + lm * g10, a01 = lp * g01 + lm * g11;
    const TW a10 = lm * g00 + lp * g10, a11 = lm * g01 + lp * g11;
    // (L B) R
    G[x + (size_t)xp * N] = a00 * rp + a01 * rm;
    G[x + (size_t)yp * N] = a00 * rm + a01 * rp;
    G[y + (size_t)xp * N] = a10 * rp + a11 * rm;
    G[y + (size_t)yp * N] = a10 * rm + a11 * rp;
  }
  __syncthreads();
}

// ---------------------------------------------------------- local updates
// Proposal decision and rank-k update (k = 1 for tU, 2 for tV and tUV).
// ratio_ss: acceptance ratio from the entries G[S,S] (get_r!).
template <int KIND, class T, class KT, class TW, class KW>
__device__ __forceinline__ double ratio_ss(Ctx<KIND, T, KT, TW, KW>& c, int lt, int o, int nv, double tu, T gxx,
                                           T gxy, T gyx, T gyy, T& r00, T& r01, T& r10, T& r11) {
  const SweepParams& P = c.P;
  double p;
  r01 = zero<T>();
  r10 = zero<T>();
  r11 = zero<T>();
  if constexpr (KIND == KDQ_TU) {
    // get_r!, src/tU/GreenMatrix.jl:49-54; γ ratio src/tU/phy_update.jl:261
    const cd Δ = reinterpret_cast<const cd*>(P.rtab)[(size_t)(lt - 1) * 16 + o * 4 + nv];
    const cd g = cvt<cd>(gxx);
    const cd pc = cd{1.0, 0.0} + Δ * (cd{1.0, 0.0} - g);
    p = abs2(pc) * P.gratio[o * 4 + nv];
    if constexpr (std::is_same_v<T, TW>) {
      if (tu < p) r00 = Δ / pc;
    } else if (tu < p) {   // only the G update uses r, in the working precision
      const cf q = cf{(float)(Δ.x * pc.x + Δ.y * pc.y), (float)(Δ.y * pc.x - Δ.x * pc.y)};
      const float inv = 1.0f / (float)abs2(pc);
      r00 = cd{q.x * inv, q.y * inv};
    }
  } else if constexpr (KIND == KDQ_TV) {
    // get_r!, src/tV/GreenMatrix.jl:76-89.  Δ = uv diag(t2) uv with
    // uv = [-h -h; -h h] is symmetric with equal diagonal entries: dd, do_
    // and 1 + dd come from the slice table, so the serial chain of a
    // proposal starts at the G-dependent products.
    const double* dt = P.dtv + ((size_t)(lt - 1) * 16 + o * 4 + nv) * 3;
    const double dd = dt[0], do_ = dt[1], dp = dt[2];
    const double Gxx = re(gxx), Gxy = re(gxy), Gyx = re(gyx), Gyy = re(gyy);
    // r = I + Δ - Δ G_SS
    const double a00 = dp - (dd * Gxx + do_ * Gyx), a01 = do_ - (dd * Gxy + do_ * Gyy);
    const double a10 = do_ - (do_ * Gxx + dd * Gyx), a11 = dp - (do_ * Gxy + dd * Gyy);
    const double det = a00 * a11 - a01 * a10;
    p = det * P.gratio[o * 4 + nv];
    if (tu < p) {   // r = r^-1 Δ = adj(r) Δ / det, needed only for the update
      const double rd = 1.0 / det;
      r00 = from_real<T>((a11 * dd - a01 * do_) * rd);
      r01 = from_real<T>((a11 * do_ - a01 * dd) * rd);
      r10 = from_real<T>((a00 * do_ - a10 * dd) * rd);
      r11 = from_real<T>((a00 * dd - a10 * do_) * rd);
    }
  } else {
    // get_r!, src/tUV/GreenMatrix.jl:73-89; weight src/tUV/phy_update.jl:193-197
    const T* t2 = reinterpret_cast<const T*>(P.rtab) + (size_t)(o * 4 + nv) * 2;
    T a00 = t2[0] - t2[0] * gxx, a01 = zero<T>() - t2[0] * gxy;
    T a10 = zero<T>() - t2[1] * gyx, a11 = t2[1] - t2[1] * gyy;
    a00 = a00 + one<T>();
    a11 = a11 + one<T>();
    const T det = a00 * a11 - a01 * a10;
    p = abs2(det) * P.gratio[o * 4 + nv] * P.xtab[o * 4 + nv];
    if (tu < p) {   // r = r^-1 Δ, needed only for the update
      const T rd = one<T>() / det;
      r00 = (a11 * rd) * t2[0];
      r01 = ((zero<T>() - a01) * rd) * t2[1];
      r10 = ((zero<T>() - a10) * rd) * t2[0];
      r11 = (a00 * rd) * t2[1];
    }
  }
  return p;
}

// Acceptance ratio p of the proposal sold -> sx (0-based o, nv) on the
// sites S = {x} (t-U) or {x, y} at slice lt, from G[S,S] (get_r!), and, when
// tu < p, r = (I + Delta (I - G_SS))^-1 Delta for the update.
template <int KIND, class T, class KT, class TW, class KW>
__device__ __forceinline__ double ratio(Ctx<KIND, T, KT, TW, KW>& c, const TW* G, int lt, int x, int y, int o,
                                        int nv, double tu, T& r00, T& r01, T& r10, T& r11) {
  const int N = c.P.Ns;
  const T gxx = cvt<T>(G[x + (size_t)x * N]);
  T gxy = zero<T>(), gyx = zero<T>(), gyy = zero<T>();
  if constexpr (KIND != KDQ_TU) {
    gxy = cvt<T>(G[x + (size_t)y * N]);
    gyx = cvt<T>(G[y + (size_t)x * N]);
    gyy = cvt<T>(G[y + (size_t)y * N]);
  }
  return ratio_ss(c, lt, o, nv, tu, gxx, gxy, gyx, gyy, r00, r01, r10, r11);
}

// ------------------------------------------------- self-learning moves (t-U)
constexpr uint32_t SLMC_STREAM = 0x534C4D43u;

__device__ inline double u53(uint32_t a, uint32_t b) {
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// Self-learning cluster moves at slice lt with G at that slice (no
// counterpart in the reference, which makes local moves only).  A move picks
// Lc consecutive sites i0 .. i0+Lc-1 (mod Ns) of the slice and runs a
// Metropolis chain of slmc_steps single-site steps on the effective weight
// W_eff(s) = exp(F(s)) prod gamma[s] (F: the convolutional effective model,
// evaluated incrementally on the 3x3 / 5x5 neighbourhoods a site change
// reaches in layers 1 and 2).  The changed sites S are then accepted together
// with probability min(1, W(s')/W(s) * W_eff(s)/W_eff(s')), which for t-U is
// |det(I + Delta_S (I - G_SS))|^2 exp(-(F(s') - F(s))): the exact FP64
// determinant ratio of the rank-|S| change (the multi-site form of get_r!,
// src/tU/GreenMatrix.jl:49-54), and on acceptance G is updated by the same
// formula as Gupdate! (src/public/Gupdate.jl:5-11) with r = M^-1 Delta_S.
// Random numbers: Philox4x32-10 on (q, sweep, chain, SLMC_STREAM) with
// q = (visit * moves + move) * (steps + 1) + step, visit = the slice's index in
// the sweep's visiting order (forward lt-1, backward 2 Nt - lt).
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void slmc_moves(Ctx<KIND, T, KT, TW, KW>& c, int lt, int visit) {
  const SweepParams& P = c.P;
  const int N = P.Ns, Nt = P.Nt, Lc = P.slmc_len, ne = P.slmc_steps;
  const int C1 = Lc + 6, C2 = Lc + 4;
  const int tid = threadIdx.x;
  unsigned char* base = c.slmc;
  const CnnW& w = *reinterpret_cast<const CnnW*>(base);
  float* a1w = reinterpret_cast<float*>(base + ((sizeof(CnnW) + 15) & ~size_t(15)));  // [7][16][C1]
  float* a2w = a1w + 7 * 16 * C1;                                                     // [5][16][C2]
  float* t1 = a2w + 5 * 16 * C2;                                                      // [9][16]
  float* t2 = t1 + 144;                                                               // [25][16]
  int* cur = reinterpret_cast<int*>(t2 + 400);
  int* orig = cur + 32;
  int* sidx = orig + 32;
  __shared__ int s_i0, s_k, s_sx, s_acc, s_m, s_bad;
  __shared__ double s_u, s_uf, s_dF;
  __shared__ T s_fm[32];
  __shared__ double s_lg;
  __shared__ cd s_ph;
  const int t0 = lt - 1;
  uint8_t* row0 = c.s + (size_t)t0 * N;
  const uint32_t sw = (uint32_t)c.ctl->sweep;
  const T* dtab = reinterpret_cast<const T*>(P.rtab) + (size_t)(lt - 1) * 16;   // Delta(old -> new)
  for (int mv = 0; mv < P.slmc_moves; ++mv) {
    const uint32_t q0 = (uint32_t)(((size_t)visit * P.slmc_moves + mv) * (size_t)(ne + 1));
    if (tid == 0) {
      const uint4 r = philox(make_uint4(q0, sw, (uint32_t)c.chain, SLMC_STREAM), (uint32_t)P.seed,
                             (uint32_t)(P.seed >> 32));
      s_i0 = (int)(((uint64_t)r.x * (uint32_t)N) >> 32);
      s_uf = u53(r.y, r.z);
      s_dF = 0.0;
    }
    __syncthreads();
    const int i0 = s_i0;
    for (int k = tid; k < Lc; k += blockDim.x) cur[k] = orig[k] = row0[wrapi(i0 + k, N)];
    __syncthreads();
    // field value at a physical (row, col), with the cluster's proposed values
    auto fld = [&](int row, int col) -> int {
      if (row == t0) {
        int kk = col - i0;
        kk += kk < 0 ? N : 0;
        if (kk < Lc) return cur[kk];
      }
      return c.s[(size_t)row * N + col];
    };
    // layer-1 window: rows t0-3 .. t0+3, columns i0-3 .. i0+Lc+2
    for (int e = tid; e < 7 * 16 * C1; e += blockDim.x) {
      const int col = e % C1, ch = (e / C1) % 16, row = e / (16 * C1);
      a1w[e] = cnn_a1(w, ch, [&](int dt, int dj) {
        return fld(wrapi(t0 - 3 + row + dt, Nt), wrapi(i0 - 3 + col + dj, N));
      });
    }
    __syncthreads();
    // layer-2 window: rows t0-2 .. t0+2, columns i0-2 .. i0+Lc+1
    for (int p = tid; p < 5 * C2; p += blockDim.x) {
      const int row = p / C2, col = p % C2;
      float z[KDQ_CNN_CH];
      cnn_z2(w, z, [&](int ch, int dt, int dj) { return a1w[((row + 1 + dt) * 16 + ch) * C1 + col + 1 + dj]; });
#pragma unroll
      for (int o = 0; o < KDQ_CNN_CH; ++o) a2w[(row * 16 + o) * C2 + col] = tanhf(z[o]);
    }
    __syncthreads();
    // Metropolis chain on the effective weight
    for (int st = 1; st <= ne; ++st) {
      if (tid == 0) {
        const uint4 r = philox(make_uint4(q0 + st, sw, (uint32_t)c.chain, SLMC_STREAM), (uint32_t)P.seed,
                               (uint32_t)(P.seed >> 32));
        const int k = (int)(((uint64_t)r.x * (uint32_t)Lc) >> 32);
        const int kv = (int)(((uint64_t)r.y * 3u) >> 32);
        const int sold = cur[k];
        s_k = k;
        s_sx = kv + (kv + 1 >= sold ? 2 : 1);
        s_u = u53(r.z, r.w);
      }
      __syncthreads();
      const int k = s_k, sx = s_sx, j = wrapi(i0 + k, N);
      // layer 1 at the 3x3 neighbourhood of (t0, j) with the new value
      if (tid < 144) {
        const int pos = tid >> 4, ch = tid & 15, dy = pos / 3, dx = pos % 3;
        const int pr = wrapi(t0 - 1 + dy, Nt), pc = wrapi(j - 1 + dx, N);
        t1[tid] = cnn_a1(w, ch, [&](int dt, int dj) {
          const int rr = wrapi(pr + dt, Nt), cc = wrapi(pc + dj, N);
          return (rr == t0 && cc == j) ? sx : fld(rr, cc);
        });
      }
      __syncthreads();
      // layer 2 at the 5x5 neighbourhood and the change of F
      double dsum = 0.0;
      for (int idx = tid; idx < 400; idx += blockDim.x) {
        const int p = idx >> 4, o = idx & 15, row = p / 5, col = k + p % 5;
        float z = w.b2[o];
        for (int ch = 0; ch < 16; ++ch)
#pragma unroll
          for (int tap = 0; tap < 9; ++tap) {
            const int ar = row + tap / 3, ac = col + tap % 3;   // layer-1 window row, column
            const bool chg = ar >= 2 && ar <= 4 && ac >= k + 2 && ac <= k + 4;
            const float v = chg ? t1[((ar - 2) * 3 + (ac - k - 2)) * 16 + ch] : a1w[(ar * 16 + ch) * C1 + ac];
            z = fmaf(w.w2f[(ch * 9 + tap) * 16 + o], v, z);
          }
        const float a = tanhf(z);
        t2[idx] = a;
        dsum += (double)w.w3s[o] * (double)(a - a2w[(row * 16 + o) * C2 + col]);
      }
      const double dF = block_sum(dsum, c.sm.red);
      if (tid == 0) {
        const int sold = cur[k];
        const double p = exp(dF) * P.gratio[(sold - 1) * 4 + sx - 1];
        const int acc = s_u < p;
        s_acc = acc;
        if (acc) {
          s_dF += dF;
          cur[k] = sx;
        }
      }
      __syncthreads();
      if (s_acc) {
        if (tid < 144) {
          const int pos = tid >> 4, ch = tid & 15;
          a1w[((2 + pos / 3) * 16 + ch) * C1 + k + 2 + pos % 3] = t1[tid];
        }
        for (int idx = tid; idx < 400; idx += blockDim.x) {
          const int p = idx >> 4, o = idx & 15;
          a2w[((p / 5) * 16 + o) * C2 + k + p % 5] = t2[idx];
        }
      }
      __syncthreads();
    }
    // the changed sites and the exact FP64 ratio
    if (tid == 0) {
      int m = 0;
      for (int k = 0; k < Lc; ++k)
        if (cur[k] != orig[k]) sidx[m++] = k;
      s_m = m;
      s_bad = 0;
      c.ctl->slmc_prop += 1;
      if (!m) c.ctl->slmc_noop += 1;
    }
    __syncthreads();
    const int m = s_m;
    if (!m) continue;
    T* M = reinterpret_cast<T*>(c.Mss);   // m x m, free between recomputes (same size as TS)
    for (int e = tid; e < m * m; e += blockDim.x) {
      const int a = e % m, b = e / m;
      const int ja = wrapi(i0 + sidx[a], N), jb = wrapi(i0 + sidx[b], N);
      const T d = dtab[(orig[sidx[a]] - 1) * 4 + cur[sidx[a]] - 1];
      T v = zero<T>() - cvt<T>(c.G[ja + (size_t)jb * N]);
      if (a == b) v = v + one<T>();
      v = d * v;
      if (a == b) v = v + one<T>();
      M[e] = v;
    }
    __syncthreads();
    gj_inverse(m, M, s_fm, c.piv, &s_bad, &s_lg, &s_ph);   // M <- M^-1, log|det M|
    if (tid == 0) {
      const double la = 2.0 * s_lg - s_dF;
      const int acc = !s_bad && isfinite(la) && s_uf < exp(la);
      s_acc = acc;
      c.ctl->slmc_acc += acc;
    }
    __syncthreads();
    if (!s_acc) continue;
    // U = G[:,S] M^-1 Delta_S (N x m) and Wr = E_S - G[S,:] (m x N)
    TW* U = c.Yw;
    TW* Wr = c.Y2w;
    for (int e = tid; e < N * m; e += blockDim.x) {
      const int i = e % N, a = e / N;
      T acc = zero<T>();
      for (int b = 0; b < m; ++b) madd(acc, cvt<T>(c.G[i + (size_t)wrapi(i0 + sidx[b], N) * N]), M[b + (size_t)a * m]);
      U[e] = cvt<TW>(acc * dtab[(orig[sidx[a]] - 1) * 4 + cur[sidx[a]] - 1]);
    }
    for (int e = tid; e < m * N; e += blockDim.x) {
      const int a = e % m, col = e / m;
      const int ja = wrapi(i0 + sidx[a], N);
      Wr[e] = (col == ja ? one<TW>() : zero<TW>()) - c.G[ja + (size_t)col * N];
    }
    __syncthreads();
    bgemm_t<Tiles<MAXRM, TW>::SM, Tiles<MAXRM, TW>::SN, TW, TW, TW, TW, true>(N, N, m, U, N, Wr, m, c.G, N);
    for (int a = tid; a < m; a += blockDim.x) row0[wrapi(i0 + sidx[a], N)] = (uint8_t)cur[sidx[a]];
    __syncthreads();
  }
}

// Fill the shared tape slice with n proposals starting at sweep-relative
// index q0 (Philox) or at the chain's explicit-tape cursor.
template <int KIND, class T, class KT, class TW, class KW>
__device__ void load_tape(Ctx<KIND, T, KT, TW, KW>& c, uint32_t q0, int n) {
  const SweepParams& P = c.P;
  if (P.tape_k) {
    const size_t base = (size_t)c.chain * P.tape_len + c.ctl->tape_pos;
    const bool ok = c.ctl->tape_pos + (size_t)n <= P.tape_len;
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
      c.tk[m] = ok ? P.tape_k[base + m] : 0;
      c.tu[m] = ok ? P.tape_u[base + m] : HUGE_VAL;   // u = +inf rejects every proposal
    }
    if (!ok && threadIdx.x == 0) atomicOr(&c.ctl->err, KDQ_FLAG_TAPE);
  } else {
    const uint32_t sw = (uint32_t)c.ctl->sweep;
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
      const uint4 r = philox(make_uint4(q0 + m, sw, (uint32_t)c.chain, TAPE_STREAM),
                             (uint32_t)P.seed, (uint32_t)(P.seed >> 32));
      c.tk[m] = (uint8_t)(((uint64_t)r.x * 3u) >> 32);
      c.tu[m] = ((double)(r.y >> 5) * 67108864.0 + (double)(r.z >> 6)) * (1.0 / 9007199254740992.0);
    }
  }
  __syncthreads();
}

template <int KIND, class T, class KT, class TW, class KW>
__device__ void finish_tape(Ctx<KIND, T, KT, TW, KW>& c, int n) {
  if (threadIdx.x == 0 && c.P.tape_k) c.ctl->tape_pos += n;
}

// All proposals of slice lt (tU, tUV) or of direction j of slice lt (tV).
// G -= u0 w0^T (+ u1 w1^T for rank 2) on the elements start, start + stride,
// ... of the column-major N x N matrix G, four independent elements per
// step so that their loads and multiply-adds overlap; with skip, entries in
// row or column x or y2 are left alone.  Per entry: v = G; v -= u0 w0;
// v -= u1 w1 (the operation order of Gupdate!, src/public/Gupdate.jl:5-11).
template <int RK, class TW>
__device__ __forceinline__ void rank_update(TW* G, int N, const TW* u0, const TW* u1, const TW* w0,
                                            const TW* w1, int start, int stride, bool skip, int x, int y2) {
  Walk w[4] = {Walk(N, N, start, 4 * stride), Walk(N, N, start + stride, 4 * stride),
               Walk(N, N, start + 2 * stride, 4 * stride), Walk(N, N, start + 3 * stride, 4 * stride)};
  while (w[0].ok()) {
    bool ok[4];
    TW v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      ok[k] = w[k].ok() && !(skip && (w[k].i == x || w[k].i == y2 || w[k].j == x || w[k].j == y2));
      v[k] = ok[k] ? G[w[k].e] : zero<TW>();
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (ok[k]) {
        madd(v[k], -u0[w[k].i], w0[w[k].j]);
        if constexpr (RK == 2) madd(v[k], -u1[w[k].i], w1[w[k].j]);
        G[w[k].e] = v[k];
      }
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) w[k].next();
  }
}

__device__ __forceinline__ double shfl_from(double v, int src) { return __shfl_sync(0xffffffffu, v, src); }
__device__ __forceinline__ cd shfl_from(cd v, int src) {
  return cd{__shfl_sync(0xffffffffu, v.x, src), __shfl_sync(0xffffffffu, v.y, src)};
}

// Sites and field index of proposal m of a layer (direction jd for t-V).
template <int KIND>
__device__ __forceinline__ void proposal_sites(const SweepParams& P, int jd, int n, int m, int& x, int& y, int& f) {
  if constexpr (KIND == KDQ_TU) {
    x = m; y = 0; f = m;
  } else if constexpr (KIND == KDQ_TV) {
    x = P.bx[jd * n + m]; y = P.by[jd * n + m]; f = jd * n + m;
  } else {
    x = P.bx[m]; y = P.by[m]; f = m;
  }
}

// FP64 local updates, a window of proposals at a time.  A rejected proposal
// leaves G unchanged, so the acceptance ratios of proposals m0, m0+1, ...
// are those a one-by-one sweep computes until the first acceptance: lane k
// of warp 0 evaluates proposal m0+k (get_r!) from the current G, the first
// accepting lane (ballot) ends the window, the proposals before it are
// rejections, and the accepted one's u' = G[:,S] r and E_S - G[S,:] are
// formed by the warp; then every thread applies G -= u' (E_S - G[S,:])
// (Gupdate!, src/public/Gupdate.jl:5-11).  The next window starts after the
// accepted proposal.  Every decision and every entry of G are bit for bit
// those of the one-by-one order; the serial FP64 ratio chain is paid once
// per accepted proposal instead of once per proposal.  Returns the index of
// the next proposal (uniform over the block); par alternates per window.
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ int propose_window(Ctx<KIND, T, KT, TW, KW>& c, TW* G, int lt, int jd, int n, int m0, int logbase,
                              uint8_t* sl, int par) {
  const SweepParams& P = c.P;
  const int N = P.Ns;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int RK = (KIND == KDQ_TU) ? 1 : 2;
  Smem<TW>& sm = c.sm;
  if (warp == 0) {
    const int W = min(32, n - m0);
    const int m = m0 + lane;
    const bool valid = lane < W;
    int x = 0, y = 0, f = 0, sx = 0, acc = 0;
    bool bad = false;
    T r00 = zero<T>(), r01 = zero<T>(), r10 = zero<T>(), r11 = zero<T>();
    if (valid) {
      proposal_sites<KIND>(P, jd, n, m, x, y, f);
      const int sold = sl[f];
      const int tk = c.tk[m];
      sx = tk + (tk + 1 >= sold ? 2 : 1);   // k-th of {1..4}\{sold}
      const double p = ratio(c, G, lt, x, y, sold - 1, sx - 1, c.tu[m], r00, r01, r10, r11);
      bad = !isfinite(p);
      acc = !bad && c.tu[m] < p;
    }
    const unsigned amask = __ballot_sync(0xffffffffu, acc);
    const int ja = amask ? __ffs(amask) - 1 : W;   // first accepting lane, W if none
    const int nres = ja < W ? ja + 1 : W;          // proposals decided by this window
    if (lane < nres && bad) atomicOr(&c.ctl->err, KDQ_FLAG_NAN);
    if (lane < nres) {
      const int logpos = logbase + m;
      if (P.acc_log && logpos >= 0 && logpos < P.acc_log_cap)
        P.acc_log[(size_t)c.chain * P.acc_log_cap + logpos] = (uint8_t)(lane == ja);
    }
    if (ja < W && lane == ja) sl[f] = (uint8_t)sx;   // lane W (no acceptance) holds no proposal
    if (ja < W) {
      const int xa = __shfl_sync(0xffffffffu, x, ja), ya = __shfl_sync(0xffffffffu, y, ja);
      const TW w00 = cvt<TW>(shfl_from(r00, ja)), w01 = cvt<TW>(shfl_from(r01, ja));
      const TW w10 = cvt<TW>(shfl_from(r10, ja)), w11 = cvt<TW>(shfl_from(r11, ja));
      for (int a = lane; a < N; a += 32) {
        const TW gx = G[a + (size_t)xa * N];
        if constexpr (RK == 1) {
          sm.ucol[0][a] = gx * w00;
        } else {
          const TW gy = G[a + (size_t)ya * N];
          sm.ucol[0][a] = gx * w00 + gy * w10;
          sm.ucol[1][a] = gx * w01 + gy * w11;
        }
        sm.wrow[0][a] = (a == xa ? one<TW>() : zero<TW>()) - G[xa + (size_t)a * N];
        if constexpr (RK == 2) sm.wrow[1][a] = (a == ya ? one<TW>() : zero<TW>()) - G[ya + (size_t)a * N];
      }
    }
    if (lane == 0) {
      sm.accept[par] = ja < W;
      sm.nxt[par] = m0 + nres;
      sm.nacc += (ja < W) ? 1 : 0;
    }
  }
  __syncthreads();
  const int next = sm.nxt[par];
  if (sm.accept[par]) {
    rank_update<RK>(G, N, sm.ucol[0], sm.ucol[1], sm.wrow[0], sm.wrow[1], tid, blockDim.x, false, 0, 0);
    __syncthreads();
  }
  c.clk.lap(1);
  return next;
}

// Delayed updates of the mixed-precision sweep (Alvarez, Loh, Scalapino,
// Comput. Phys. Commun. 179, 2008; no counterpart in the reference, which
// updates G after every acceptance, src/public/Gupdate.jl:5-11).  The rank-1
// (t-U) or rank-2 (t-V, t-UV) changes of accepted proposals are kept as
// vector pairs u_q = (G[:,S] r)_q, w_q = (E_S - G[S,:])_q in shared memory,
// the current Green's function being G - sum_q u_q w_q^T; a proposal's
// ratio and an accepted proposal's new vectors read G through that sum, and
// G itself is rewritten once per KDQ_DELAY vectors (delayed_flush) instead
// of once per acceptance: the N x N matrix streams through L2 KDQ_DELAY / k
// times less often.  Decisions use the same windows as the FP64 sweep.  16
// vectors (48 KB of shared memory at the largest lattice) keep two CTAs per
// SM; the flush's cost is mostly its pass over G, so 16 instead of 8 nearly
// halves it while the correction sums of the windows grow by 4 terms on
// average.
#define KDQ_DELAY 16
template <class TW>
struct Delay {
  TW U[KDQ_DELAY][KDQ_MAX_NS];
  TW W[KDQ_DELAY][KDQ_MAX_NS];
  TW diag[KDQ_MAX_NS];   // diagonal of the stored G (refreshed at slice start and after each flush)
};

// G -= sum_{q < kd} U[q] W[q]^T.  Complex G: one N x N x kd product on the
// tensor pipe (3xTF32, FP32 accumulators starting from G).  Otherwise warps
// own columns, lanes rows, in sequential FMAs.
template <class TW>
__device__ void delayed_flush(TW* G, int N, const Delay<TW>& db, int kd) {
  if constexpr (std::is_same_v<TW, cf>) {
    tc_zgemm<2, 2, true, true>(N, N, kd, reinterpret_cast<const float*>(&db.U[0][0]), KDQ_MAX_NS,
                               reinterpret_cast<const float*>(&db.W[0][0]), KDQ_MAX_NS, G, N);
    return;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int b = warp; b < N; b += nw) {
    TW wb[KDQ_DELAY];
#pragma unroll
    for (int q = 0; q < KDQ_DELAY; ++q) wb[q] = q < kd ? db.W[q][b] : zero<TW>();
    TW* col = G + (size_t)b * N;
    for (int a = lane; a < N; a += 32) {
      TW v = col[a];
#pragma unroll
      for (int q = 0; q < KDQ_DELAY; ++q)
        if (q < kd) madd(v, -db.U[q][a], wb[q]);
      col[a] = v;
    }
  }
  __syncthreads();
}

// (G - U W)[i, j] for the kd pending vector pairs
template <class TW>
__device__ __forceinline__ TW delayed_entry(const TW* G, int N, const Delay<TW>& db, int kd, int i, int j) {
  TW v = G[i + (size_t)j * N];
  for (int q = 0; q < kd; ++q) madd(v, -db.U[q][i], db.W[q][j]);
  return v;
}

// (G - U W)[i, i] from the shared-memory copy of G's diagonal
template <class TW>
__device__ __forceinline__ TW delayed_diag(const TW* gdiag, const Delay<TW>& db, int kd, int i) {
  TW v = gdiag[i];
  for (int q = 0; q < kd; ++q) madd(v, -db.U[q][i], db.W[q][i]);
  return v;
}

// Copies the diagonal of the stored G into shared memory (all threads call it).
template <class TW>
__device__ __forceinline__ void load_gdiag(TW* gdiag, const TW* G, int N) {
  for (int a = threadIdx.x; a < N; a += blockDim.x) gdiag[a] = G[a + (size_t)a * N];
  __syncthreads();
}

// One window of proposals with delayed updates; kd (uniform over the CTA)
// is the number of pending vector pairs.  Returns the next proposal index.
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ int propose_window_delayed(Ctx<KIND, T, KT, TW, KW>& c, TW* G, int lt, int jd, int n, int m0,
                                      int logbase, uint8_t* sl, int par, Delay<TW>& db, int& kd) {
  const SweepParams& P = c.P;
  const int N = P.Ns;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int RK = (KIND == KDQ_TU) ? 1 : 2;
  Smem<TW>& sm = c.sm;
  if (warp == 0) {
    const int W = min(32, n - m0);
    const int m = m0 + lane;
    const bool valid = lane < W;
    int x = 0, y = 0, f = 0, sx = 0, acc = 0;
    bool bad = false;
    T r00 = zero<T>(), r01 = zero<T>(), r10 = zero<T>(), r11 = zero<T>();
    if (valid) {
      proposal_sites<KIND>(P, jd, n, m, x, y, f);
      const int sold = sl[f];
      const int tk = c.tk[m];
      sx = tk + (tk + 1 >= sold ? 2 : 1);   // k-th of {1..4}\{sold}
      const T gxx = cvt<T>(delayed_diag(db.diag, db, kd, x));
      T gxy = zero<T>(), gyx = zero<T>(), gyy = zero<T>();
      if constexpr (RK == 2) {
        gxy = cvt<T>(delayed_entry(G, N, db, kd, x, y));
        gyx = cvt<T>(delayed_entry(G, N, db, kd, y, x));
        gyy = cvt<T>(delayed_diag(db.diag, db, kd, y));
      }
      const double p = ratio_ss(c, lt, sold - 1, sx - 1, c.tu[m], gxx, gxy, gyx, gyy, r00, r01, r10, r11);
      bad = !isfinite(p);
      acc = !bad && c.tu[m] < p;
    }
    const unsigned amask = __ballot_sync(0xffffffffu, acc);
    const int ja = amask ? __ffs(amask) - 1 : W;   // first accepting lane, W if none
    const int nres = ja < W ? ja + 1 : W;          // proposals decided by this window
    if (lane < nres && bad) atomicOr(&c.ctl->err, KDQ_FLAG_NAN);
    if (lane < nres) {
      const int logpos = logbase + m;
      if (P.acc_log && logpos >= 0 && logpos < P.acc_log_cap)
        P.acc_log[(size_t)c.chain * P.acc_log_cap + logpos] = (uint8_t)(lane == ja);
    }
    if (ja < W && lane == ja) {
      sl[f] = (uint8_t)sx;   // lane W (no acceptance) holds no proposal
      sm.site[0] = x;
      sm.site[1] = y;
      sm.rr[0] = cvt<TW>(r00);
      sm.rr[1] = cvt<TW>(r01);
      sm.rr[2] = cvt<TW>(r10);
      sm.rr[3] = cvt<TW>(r11);
    }
    if (lane == 0) {
      sm.accept[par] = ja < W;
      sm.nxt[par] = m0 + nres;
      sm.nacc += (ja < W) ? 1 : 0;
    }
  }
  __syncthreads();
  c.clk.lap(7);   // the window's decision (ratios, ballot, publication)
  const int next = sm.nxt[par];
  if (sm.accept[par]) {
    // the accepted proposal's vectors from the current G (= G - U W)
    const int xa = sm.site[0], ya = sm.site[1];
    const TW w00 = sm.rr[0], w01 = sm.rr[1], w10 = sm.rr[2], w11 = sm.rr[3];
    for (int a = tid; a < N; a += blockDim.x) {
      const TW gx = delayed_entry(G, N, db, kd, a, xa);
      const TW rx = delayed_entry(G, N, db, kd, xa, a);
      if constexpr (RK == 1) {
        db.U[kd][a] = gx * w00;
        db.W[kd][a] = (a == xa ? one<TW>() : zero<TW>()) - rx;
      } else {
        const TW gy = delayed_entry(G, N, db, kd, a, ya);
        const TW ry = delayed_entry(G, N, db, kd, ya, a);
        db.U[kd][a] = gx * w00 + gy * w10;
        db.U[kd + 1][a] = gx * w01 + gy * w11;
        db.W[kd][a] = (a == xa ? one<TW>() : zero<TW>()) - rx;
        db.W[kd + 1][a] = (a == ya ? one<TW>() : zero<TW>()) - ry;
      }
    }
    __syncthreads();
    kd += RK;
    if (kd + RK > KDQ_DELAY) {   // no room for another acceptance
      delayed_flush(G, N, db, kd);
      load_gdiag(db.diag, G, N);
      kd = 0;
    }
  }
  c.clk.lap(1);
  return next;
}

template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void update_layer(Ctx<KIND, T, KT, TW, KW>& c, int lt, int j, bool fwd) {
  const SweepParams& P = c.P;
  const int Nt = P.Nt, pf = P.n_field;
  uint8_t* sl = c.s + (size_t)(lt - 1) * pf;
  // sweep-relative index of the first proposal of this slice
  const uint32_t qs = fwd ? (uint32_t)(lt - 1) * pf : (uint32_t)(Nt + (Nt - lt)) * pf;
  int n, off;
  if constexpr (KIND == KDQ_TV) {
    n = P.Ns / 2;
    off = (fwd ? (P.z - 1 - j) : j) * n;
  } else {
    n = pf;
    off = 0;
  }
  load_tape(c, qs + off, n);
  const int logbase = (int)(c.ctl->log_pos);
  // the slice's fields and acceptance count live in shared memory while its
  // windows run (a window's decision then waits on no global round trip)
  uint8_t* fs = c.sm.fld;
  for (int e = threadIdx.x; e < pf; e += blockDim.x) fs[e] = sl[e];
  if (threadIdx.x == 0) c.sm.nacc = 0;
  __syncthreads();
  int par = 0;
  if constexpr (std::is_same_v<T, TW>) {
    for (int m = 0; m < n; par ^= 1) m = propose_window<MAXRM>(c, c.G, lt, j, n, m, logbase, fs, par);
  } else {
    __shared__ Delay<TW> db;
    int kd = 0;
    load_gdiag(db.diag, c.G, P.Ns);
    for (int m = 0; m < n; par ^= 1) m = propose_window_delayed<MAXRM>(c, c.G, lt, j, n, m, logbase, fs, par, db, kd);
    if (kd) delayed_flush(c.G, P.Ns, db, kd);
  }
  __syncthreads();
  for (int e = threadIdx.x; e < pf; e += blockDim.x) sl[e] = fs[e];
  if (threadIdx.x == 0) {
    c.ctl->log_pos += n;
    c.ctl->n_prop += n;
    c.ctl->n_acc += c.sm.nacc;
  }
  finish_tape(c, n);
  __syncthreads();
}

// --------------------------------------------------------- stabilisation
// Thin-factor block products: instead of forming BM = B_n ... B_m (N x N)
// and multiplying it into BR (the reference's BM_F! + mul!), the slices are
// applied directly to the N x ns factor (left) or the ns x N factor (right);
// same product, half the multiply-adds.

// Y (N x ns) <- B_lt Y, ping-ponging with Y2; returns the buffer holding it.
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ TW* apply_slice_left(Ctx<KIND, T, KT, TW, KW>& c, TW* Y, TW* Y2, int lt) {
  const SweepParams& P = c.P;
  const int N = P.Ns, ns = N / 2;
  if constexpr (KIND == KDQ_TV) {
    gemm_thin<MAXRM, TW>(N, ns, N, c.eK, N, Y, N, Y2, N);
    for (int j = P.z - 1; j >= 0; --j) {
      tv_coeffs(c, lt, j, +1);
      const TW* L = c.sm.dvec;
      for (int e = threadIdx.x; e < (N / 2) * ns; e += blockDim.x) {
        const int i = e % (N / 2), col = e / (N / 2);
        const int x = P.bx[j * (N / 2) + i], y = P.by[j * (N / 2) + i];
        const TW lp = L[2 * i], lm = L[2 * i + 1];
        const TW vx = Y2[x + (size_t)col * N], vy = Y2[y + (size_t)col * N];
        Y2[x + (size_t)col * N] = lp * vx + lm * vy;
        Y2[y + (size_t)col * N] = lm * vx + lp * vy;
      }
      __syncthreads();
    }
  } else {
    slice_diag(c, lt, +1);
    kmul_left<MAXRM, true>(N, ns, N, c.eK, kin_frag(c.P, KIN_EK, 0), N, Y, N, Y2, N, c.sm.dvec);
  }
  return Y2;
}

// Z (ns x N) <- Z B_lt, ping-ponging with Z2; returns the buffer holding it.
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ TW* apply_slice_right(Ctx<KIND, T, KT, TW, KW>& c, TW* Z, TW* Z2, int lt) {
  const SweepParams& P = c.P;
  const int N = P.Ns, ns = N / 2;
  if constexpr (KIND == KDQ_TV) {
    for (int j = 0; j < P.z; ++j) {        // Z V_1 V_2 ... V_z, V_j = L (symmetric)
      tv_coeffs(c, lt, j, +1);
      const TW* L = c.sm.dvec;
      for (int e = threadIdx.x; e < ns * (N / 2); e += blockDim.x) {
        const int row = e % ns, i = e / ns;
        const int x = P.bx[j * (N / 2) + i], y = P.by[j * (N / 2) + i];
        const TW lp = L[2 * i], lm = L[2 * i + 1];
        const TW vx = Z[row + (size_t)x * ns], vy = Z[row + (size_t)y * ns];
        Z[row + (size_t)x * ns] = vx * lp + vy * lm;
        Z[row + (size_t)y * ns] = vx * lm + vy * lp;
      }
      __syncthreads();
    }
    gemm_thin<MAXRM, TW>(ns, N, N, Z, ns, c.eK, N, Z2, ns);
  } else {
    slice_diag(c, lt, +1);
    for (int e = threadIdx.x; e < ns * N; e += blockDim.x) {
      const int col = e / ns;
      Z[e] = Z[e] * c.sm.dvec[col];
    }
    __syncthreads();
    kmul_right<MAXRM, true>(ns, N, N, Z, ns, c.eK, kin_frag(c.P, KIN_EK, 1), N, Z2, ns);
  }
  return Z2;
}

// log|det| and phase of the triangular factors dropped from one side of a
// chain's B-chain up to node k (side 0: BLs, 1: BRs).
__device__ inline double* lw_at(const SweepParams& P, int chain, int side, int k) {
  return P.lw + ((size_t)chain * 2 * P.NN + (size_t)side * P.NN + (k - 1)) * 3;
}

// G = I - BR (BL BR)^-1 BL (get_G!, src/public/Gupdate.jl:139-157); records
// the drift against the wrapped G when `drift` is set.  BL, BR are the
// factors at node `node` (1-based): with the dropped factors of both sides
// the pivots of (BL BR) give log|det(P^H B(Theta,0) P)| of the current
// fields, kept in ChainCtl (no counterpart in the reference, which discards
// the R factors).
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void get_G(Ctx<KIND, T, KT, TW, KW>& c, const typename Ctx<KIND, T, KT, TW, KW>::TS* BL,
                      const typename Ctx<KIND, T, KT, TW, KW>::TS* BR, bool drift, int node) {
  using TS = typename Ctx<KIND, T, KT, TW, KW>::TS;
  const int N = c.P.Ns, ns = N / 2;
  gemm_thin<MAXRM, TS>(ns, ns, N, BL, ns, BR, N, c.Mss, ns);
  __shared__ int bad;
  __shared__ TS fcol[KDQ_MAX_NS / 2];
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  // (BL BR)^-1 by Gauss-Jordan, then X = (BL BR)^-1 BL and BR X as block GEMMs
  // (the reference solves with getrf + getrs; the product is the same)
  __shared__ double mlg;   // written and read by thread 0 only
  __shared__ cd mph;
  gj_inverse(ns, c.Mss, fcol, c.piv, &bad, &mlg, &mph);
  if (threadIdx.x == 0) {
    const double* l = lw_at(c.P, c.chain, 0, node);
    const double* r = lw_at(c.P, c.chain, 1, node);
    const cd ph = mph * mkc(l[1], l[2]) * mkc(r[1], r[2]);
    c.ctl->logdet = mlg + l[0] + r[0];
    c.ctl->det_re = ph.x;
    c.ctl->det_im = ph.y;
  }
  double d2 = 0.0, n2 = 0.0;
  if constexpr (std::is_same_v<TS, cdf>) {
    // Mixed sweep: (BL BR) and its inverse in double-float set the
    // conditioning; the two products after them feed the FP32 G, so they run
    // as complex 3xTF32 tensor tiles to FP32 accuracy (X and BR X in FP32,
    // in the first halves of the X and Gd buffers).
    cf* Xf = reinterpret_cast<cf*>(c.X);
    cf* Gf = reinterpret_cast<cf*>(c.Gd);
    tc_zgemm<4, 4>(ns, N, ns, reinterpret_cast<const float*>(c.Mss), ns, reinterpret_cast<const float*>(BL), ns,
                   Xf, ns);
    tc_zgemm<4, 2>(N, N, ns, reinterpret_cast<const float*>(BR), N, reinterpret_cast<const float*>(Xf), ns, Gf, N);
    for (Walk w(N, N); w.ok(); w.next()) {
      const cf p = Gf[w.e];
      const cf g = cf{(w.i == w.j ? 1.0f : 0.0f) - p.x, -p.y};
      if (drift) {
        const cf o = c.G[w.e];
        const double dx = (double)o.x - (double)g.x, dy = (double)o.y - (double)g.y;
        d2 += dx * dx + dy * dy;
        n2 += (double)g.x * g.x + (double)g.y * g.y;
      }
      c.G[w.e] = g;
    }
  } else {
    gemm_thin<MAXRM, TS>(ns, N, ns, c.Mss, ns, BL, ns, c.X, ns);
    gemm_sq<MAXRM, TS>(N, N, ns, BR, N, c.X, ns, c.Gd, N);
    for (Walk w(N, N); w.ok(); w.next()) {
      TS g = zero<TS>() - c.Gd[w.e];
      if (w.i == w.j) g = g + one<TS>();
      if (drift) {
        d2 += abs2(cvt<TS>(c.G[w.e]) - g);
        n2 += abs2(g);
      }
      c.G[w.e] = cvt<TW>(g);
    }
  }
  if (drift) {
    d2 = block_sum(d2, c.sm.red);
    n2 = block_sum(n2, c.sm.red);
    if (threadIdx.x == 0) {
      const double dr = sqrt(d2 / n2);
      if (c.ctl->drift_pos < c.P.drift_cap)
        c.P.drift[(size_t)c.chain * c.P.drift_cap + c.ctl->drift_pos] = dr;
      c.ctl->drift_pos += 1;
      c.ctl->n_recompute += 1;
      if (!(dr <= c.ctl->max_drift)) c.ctl->max_drift = isfinite(dr) ? fmax(dr, c.ctl->max_drift) : dr;
    }
  }
  if (threadIdx.x == 0 && bad) atomicOr(&c.ctl->err, KDQ_FLAG_SINGULAR);
  __syncthreads();
}

// Thin Q of the N x ns block product A (destroyed) into Q, and the log|det|
// and phase of the dropped triangle.  Plain sweep: Householder (the
// reference's ?geqrf + ?orgqr).  Mixed sweep: one-pass Cholesky QR in
// double-float arithmetic, W = A^H A = R^H R, Q = A R^-1 (GEMM-shaped, about a
// third of the Householder's operations): the mixed sweep's slice matrices
// D eK have unitary D, so cond(A) <= cond(eK)^n_wrap and the loss of
// orthogonality, ~cond(A)^2 2^-48, stays far below the FP32 G it feeds (2e-12
// at t-U 12x12, n_wrap 8); when a pivot reveals cond(A)^2 > 1e8 the
// Householder form runs instead.  The span, and so G, is the same either way
// (Q differs by a unitary column rotation).  scratch: N x ns (TS).
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void thin_q(Ctx<KIND, T, KT, TW, KW>& c, typename Ctx<KIND, T, KT, TW, KW>::TS* A,
                       typename Ctx<KIND, T, KT, TW, KW>::TS* Q, typename Ctx<KIND, T, KT, TW, KW>::TS* scratch,
                       double* qlg, cd* qph) {
  using TS = typename Ctx<KIND, T, KT, TW, KW>::TS;
  const int N = c.P.Ns, ns = N / 2;
  if constexpr (!std::is_same_v<T, TW>) {
    __shared__ int bad;
    __shared__ double rinv[KDQ_MAX_NS / 2];
    if (threadIdx.x == 0) bad = 0;
    for (size_t e = threadIdx.x; e < (size_t)N * ns; e += blockDim.x) {   // A^H (ns x N)
      const int i = e % N, col = e / N;
      scratch[col + (size_t)i * ns] = conjg(A[e]);
    }
    __syncthreads();
    gemm_thin<MAXRM, TS>(ns, ns, N, scratch, ns, A, N, c.Mss, ns);
    chol_upper(ns, c.Mss, 1e-8, rinv, &bad, qlg);
    if (!bad) {
      trsm_right_upper(N, ns, A, c.Mss, rinv, Q);
      if (threadIdx.x == 0) *qph = mkc(1.0, 0.0);
      __syncthreads();
      return;
    }
  }
  householder_q(N, ns, A, Q, c.sm.wn, c.sm.red, qlg, qph);
}

// BRs[k+1] = orth_cols(BM(k) BRs[k]) then G recompute at node k+1.
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void node_forward(Ctx<KIND, T, KT, TW, KW>& c, int k) {
  using TS = typename Ctx<KIND, T, KT, TW, KW>::TS;
  const SweepParams& P = c.P;
  const int N = P.Ns, ns = N / 2;
  const size_t fs = (size_t)N * ns;
  TS* BRk = P.BRs<TS>(c.chain) + (size_t)(k - 1) * fs;
  TS* BRn = BRk + fs;
  for (size_t e = threadIdx.x; e < fs; e += blockDim.x) c.Yw[e] = cvt<TW>(BRk[e]);
  __syncthreads();
  TW* cur = c.Yw;
  TW* oth = c.Y2w;
  for (int lt = (int)P.nodes[k - 1] + 1; lt <= (int)P.nodes[k]; ++lt) {
    TW* res = apply_slice_left<MAXRM>(c, cur, oth, lt);
    oth = cur;
    cur = res;
  }
  TS* src;
  if constexpr (std::is_same_v<T, TW>) {
    src = cur;
  } else {   // the block product in working precision, its QR in double-float
    for (size_t e = threadIdx.x; e < fs; e += blockDim.x) c.Y[e] = cvt<TS>(cur[e]);
    __syncthreads();
    src = c.Y;
  }
  c.clk.lap(3);
  __shared__ double qlg;   // written and read by thread 0 only
  __shared__ cd qph;
  thin_q<MAXRM>(c, src, BRn, c.Y2, &qlg, &qph);
  if (threadIdx.x == 0) {   // B(tau_{k+1}, 0) P = BRs[k+1] R_{k+1} ... R_1
    const double* a = lw_at(P, c.chain, 1, k);
    double* b = lw_at(P, c.chain, 1, k + 1);
    const cd ph = mkc(a[1], a[2]) * qph;
    b[0] = a[0] + qlg;
    b[1] = ph.x;
    b[2] = ph.y;
  }
  c.clk.lap(4);
  const TS* BLn = P.BLs<TS>(c.chain) + (size_t)k * fs;
  get_G<MAXRM>(c, BLn, BRn, true, k + 1);
  c.clk.lap(5);
  if (threadIdx.x == 0) c.ctl->idx = k + 1;
}

// BLs[k] = orth_rows(BLs[k+1] BM(k)) then (optionally) G recompute.
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void node_backward(Ctx<KIND, T, KT, TW, KW>& c, int k, bool recompute, bool drift) {
  using TS = typename Ctx<KIND, T, KT, TW, KW>::TS;
  const SweepParams& P = c.P;
  const int N = P.Ns, ns = N / 2;
  const size_t fs = (size_t)N * ns;
  TS* BLk = P.BLs<TS>(c.chain) + (size_t)(k - 1) * fs;
  const TS* BLn = BLk + fs;
  for (size_t e = threadIdx.x; e < fs; e += blockDim.x) c.Yw[e] = cvt<TW>(BLn[e]);
  __syncthreads();
  TW* cur = c.Yw;
  TW* oth = c.Y2w;
  for (int lt = (int)P.nodes[k]; lt > (int)P.nodes[k - 1]; --lt) {
    TW* res = apply_slice_right<MAXRM>(c, cur, oth, lt);
    oth = cur;
    cur = res;
  }
  // orth_rows: QR of Z^H (N x ns) in the stabilisation type, BL = Q^H
  TS* A;
  TS* Q;
  if constexpr (std::is_same_v<T, TW>) {
    A = oth;
    Q = cur;
  } else {
    A = c.Y;
    Q = c.Y2;
  }
  for (size_t e = threadIdx.x; e < fs; e += blockDim.x) {
    const int r = e % ns, col = e / ns;
    A[col + (size_t)r * N] = conjg(cvt<TS>(cur[e]));
  }
  __syncthreads();
  c.clk.lap(3);
  __shared__ double qlg;   // written and read by thread 0 only
  __shared__ cd qph;
  thin_q<MAXRM>(c, A, Q, c.X, &qlg, &qph);
  for (size_t e = threadIdx.x; e < fs; e += blockDim.x) {
    const int r = e % ns, col = e / ns;
    BLk[e] = conjg(Q[col + (size_t)r * N]);
  }
  if (threadIdx.x == 0) {   // P^H B(Theta, tau_k) = R_k^H ... BLs[k]: the factor is R^H
    const double* a = lw_at(P, c.chain, 0, k + 1);
    double* b = lw_at(P, c.chain, 0, k);
    const cd ph = mkc(a[1], a[2]) * conjg(qph);
    b[0] = a[0] + qlg;
    b[1] = ph.x;
    b[2] = ph.y;
  }
  __syncthreads();
  c.clk.lap(4);
  if (recompute) get_G<MAXRM>(c, BLk, P.BRs<TS>(c.chain) + (size_t)(k - 1) * fs, drift, k);
  c.clk.lap(5);
  if (threadIdx.x == 0) c.ctl->idx = k;
}

// ------------------------------------------------------------ measurement
// At t0 = Nt/2 the current G is the equal-time Green's function at the
// middle of the projection, which the Rényi-2 Grover determinant of replica
// pairs is evaluated on; keep an FP64 copy when the caller asked for it.
template <int KIND, class T, class KT, class TW, class KW>
__device__ void keep_middle(Ctx<KIND, T, KT, TW, KW>& c, int t0) {
  const SweepParams& P = c.P;
  if (!P.gmid || 2 * t0 != P.Nt) return;
  T* dst = static_cast<T*>(P.gmid) + (size_t)c.chain * P.sz_NN;
  for (int e = threadIdx.x; e < P.Ns * P.Ns; e += blockDim.x) dst[e] = cvt<T>(c.G[e]);
  __syncthreads();
}

__device__ inline double re_prod(double k, double g) { return k * g; }
__device__ inline double re_prod(double k, cd g) { return k * g.x; }
__device__ inline double re_prod(cd k, cd g) { return k.x * g.x - k.y * g.y; }

template <int KIND, class T, class KT, class TW, class KW>
__device__ void observables(Ctx<KIND, T, KT, TW, KW>& c, const TW* G0);

// Equal-time observables at tau = Nt/2 from G at slice t0 (phy_measure):
// wrap a copy to Nt/2, symmetrise with HalfeK, accumulate one row.
// tU: src/tU/phy_update.jl:154-254; tV: src/tV/phy_update.jl:207-314;
// tUV: src/tUV/phy_update.jl:205-355.  The honeycomb structure factors keep
// the reference's accumulation (only the first term of each correlator in
// the complex branch, where the `+adjoint(...)` lines are discarded
// statements); `xy_i` is called with its real three-argument signature.
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void measure(Ctx<KIND, T, KT, TW, KW>& c, int t0) {
  const SweepParams& P = c.P;
  keep_middle(c, t0);
  const int N = P.Ns, Nt = P.Nt, half = Nt / 2;
  TW* G0 = c.W2;
  TW* W = c.W1;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) G0[e] = c.G[e];
  __syncthreads();
  if (2 * t0 > Nt) {
    for (int t = t0; t > half; --t) {
      if constexpr (KIND == KDQ_TV) {
        for (int j = 0; j < P.z; ++j) tv_rotate(c, G0, t, j, -1);
        gemm_sq<MAXRM, TW>(N, N, N, c.eKinv, N, G0, N, W, N);
        gemm_sq<MAXRM, TW>(N, N, N, W, N, c.eK, N, G0, N);
      } else {
        wrap_bwd_kv<MAXRM>(c, G0, W, t);
      }
    }
  } else {
    for (int t = t0 + 1; t <= half; ++t) {
      if constexpr (KIND == KDQ_TV) {
        gemm_sq<MAXRM, TW>(N, N, N, G0, N, c.eKinv, N, W, N);
        gemm_sq<MAXRM, TW>(N, N, N, c.eK, N, W, N, G0, N);
        for (int j = P.z - 1; j >= 0; --j) tv_rotate(c, G0, t, j, +1);
      } else {
        wrap_fwd_kv<MAXRM>(c, G0, W, t);
      }
    }
  }
  kmul_left<MAXRM, false>(N, N, N, c.HalfeK, kin_frag(c.P, KIN_HALFEK, 0), N, G0, N, W, N);
  kmul_right<MAXRM, false>(N, N, N, W, N, c.HalfeKinv, kin_frag(c.P, KIN_HALFEKINV, 1), N, G0, N);
  observables(c, G0);
}

// Observables of the symmetrised Green's function G0 at tau = Nt/2,
// accumulated into the chain's current measurement row.
template <int KIND, class T, class KT, class TW, class KW>
__device__ void observables(Ctx<KIND, T, KT, TW, KW>& c, const TW* G0) {
  const SweepParams& P = c.P;
  const int N = P.Ns;
  double acc[KDQ_MAX_OBS];
#pragma unroll
  for (int q = 0; q < KDQ_MAX_OBS; ++q) acc[q] = 0.0;
  // kinetic energy: Σ K .* G0
  double ek = 0.0;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) ek += re_prod(c.Kmat[e], cvt<T>(G0[e]));
  // on-site term
  double eu = 0.0;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const T d = cvt<T>(G0[i + (size_t)i * N]);
    if constexpr (KIND == KDQ_TUV && sizeof(T) == sizeof(double)) {
      eu += re((one<T>() - d) * (one<T>() - d));
    } else {
      eu += re((one<T>() - d) * conjg(d));
    }
  }
  // bond term
  double ev = 0.0;
  if constexpr (KIND != KDQ_TU) {
    const int nbond = KIND == KDQ_TV ? (N / 2) * P.z : N * P.z;
    for (int b = threadIdx.x; b < nbond; b += blockDim.x) {
      const int x = P.bx[b], y = P.by[b];
      const T gxx = cvt<T>(G0[x + (size_t)x * N]), gyy = cvt<T>(G0[y + (size_t)y * N]);
      const T gxy = cvt<T>(G0[x + (size_t)y * N]), gyx = cvt<T>(G0[y + (size_t)x * N]);
      const T ox = one<T>() - gxx, oy = one<T>() - gyy;
      if constexpr (KIND == KDQ_TV || sizeof(T) == sizeof(double)) {
        const double v = re(ox * oy - gxy * gyx);
        ev += KIND == KDQ_TV ? v : 2.0 * v + 2.0 * re(oy * ox);
      } else {
        ev += re(ox * oy - gxy * gyx) + re(conjg(gxx * gyy - gxy * gyx)) + re(oy * conjg(gxx)) +
              re(ox * conjg(gyy));
      }
    }
  }
  // honeycomb structure factors over (displacement, cell) pairs
  double sf[8];
#pragma unroll
  for (int q = 0; q < 8; ++q) sf[q] = 0.0;
  const bool hc = P.lattice == KDQ_HONEYCOMB120 || P.lattice == KDQ_HONEYCOMB60;
  if (hc) {
    const int L1 = P.L1, L2 = P.L2, nc = L1 * L2;
    for (int e = threadIdx.x; e < nc * nc; e += blockDim.x) {
      const int r = e / nc, cell = e % nc;
      const int rx = r % L1 + 1, ry = r / L1 + 1;
      const int ix = cell % L1 + 1, iy = cell / L1 + 1;
      const int jx = (ix + rx - 1) % L1 + 1, jy = (iy + ry - 1) % L2 + 1;
      const int a1 = 2 * (ix + (iy - 1) * L1) - 2, a2 = 2 * (jx + (jy - 1) * L1) - 2;
      const int b1 = a1 + 1, b2 = a2 + 1;
      const double ph = P.cosr[r];
      auto g = [&](int i, int j) { return cvt<T>(G0[i + (size_t)j * N]); };
      const T o = one<T>();
      if constexpr (KIND == KDQ_TV) {
        double t[4];
        if (a1 == a2) {
          t[0] = re(o - g(a1, a1));
          t[1] = re(o - g(b1, b1));
        } else {
          t[0] = re((o - g(a1, a1)) * (o - g(a2, a2)) - g(a1, a2) * g(a2, a1));
          t[1] = re((o - g(b1, b1)) * (o - g(b2, b2)) - g(b1, b2) * g(b2, b1));
        }
        t[2] = re((o - g(b1, b1)) * (o - g(a2, a2)) - g(b1, a2) * g(a2, b1));
        t[3] = re((o - g(a1, a1)) * (o - g(b2, b2)) - g(a1, b2) * g(b2, a1));
#pragma unroll
        for (int q = 0; q < 4; ++q) { sf[q] += t[q]; sf[4 + q] += ph * t[q]; }
      } else {
        const T del = a1 == a2 ? o : zero<T>();
        double t1, t2;
        if constexpr (KIND == KDQ_TUV && sizeof(T) == sizeof(double)) {
          t1 = 2 * re((o - g(a1, a1)) * (o - g(a2, a2)) + (del - g(a1, a2)) * g(a2, a1)) +
               2 * re((o - g(b1, b1)) * (o - g(b2, b2)) + (del - g(b1, b2)) * g(b2, b1)) -
               2 * re((o - g(b1, b1)) * (o - g(a2, a2)) - g(b1, a2) * g(a2, b1)) -
               2 * re((o - g(a1, a1)) * (o - g(b2, b2)) - g(a1, b2) * g(b2, a1));
          t2 = 2 * re((o - g(a1, a1)) * (o - g(a2, a2))) + 2 * re((o - g(b1, b1)) * (o - g(b2, b2))) -
               2 * re((o - g(b1, b1)) * (o - g(a2, a2))) - 2 * re((o - g(a1, a1)) * (o - g(b2, b2)));
        } else {
          t1 = re((o - g(a1, a1)) * (o - g(a2, a2)) + (del - g(a1, a2)) * g(a2, a1)) +
               re((o - g(b1, b1)) * (o - g(b2, b2)) + (del - g(b1, b2)) * g(b2, b1)) -
               re((o - g(b1, b1)) * (o - g(a2, a2)) - g(b1, a2) * g(a2, b1)) -
               re((o - g(a1, a1)) * (o - g(b2, b2)) - g(a1, b2) * g(b2, a1));
          t2 = re((o - g(a1, a1)) * conjg(g(a2, a2))) + re((o - g(b1, b1)) * conjg(g(b2, b2))) -
               re((o - g(a1, a1)) * conjg(g(b2, b2))) - re((o - g(b1, b1)) * conjg(g(a2, a2)));
          if (P.meas_full) {   // the discarded adjoint (opposite-spin) terms restored
            const double u1 = t1 + re(conjg(g(a1, a1) * g(a2, a2) + g(a1, a2) * (del - g(a2, a1)))) +
                              re(conjg(g(b1, b1) * g(b2, b2) + g(b1, b2) * (del - g(b2, b1)))) -
                              re(conjg(g(b1, b1) * g(a2, a2) - g(b1, a2) * g(a2, b1))) -
                              re(conjg(g(a1, a1) * g(b2, b2) - g(a1, b2) * g(b2, a1)));
            const double u2 = t2 + re(conjg(g(a1, a1)) * (o - g(a2, a2))) + re(conjg(g(b1, b1)) * (o - g(b2, b2))) -
                              re(conjg(g(a1, a1)) * (o - g(b2, b2))) - re(conjg(g(b1, b1)) * (o - g(a2, a2)));
            sf[4] += u1 + u2;
            sf[5] += ph * (u1 + u2);
            sf[6] += u1 - u2;
            sf[7] += ph * (u1 - u2);
          }
        }
        sf[0] += t1 + t2;
        sf[1] += ph * (t1 + t2);
        sf[2] += t1 - t2;
        sf[3] += ph * (t1 - t2);
      }
    }
  } else if constexpr (KIND != KDQ_TV) {
    // square lattices (t-U, complex t-UV, full measurement only): the
    // staggered charge and spin structure factors at (pi, pi),
    // sum_ij e_i e_j <rho_i rho_j> with every term of the honeycomb
    // correlators above (no counterpart in the reference, whose square
    // branch measures none); e = the lattice's two-colouring
    if (P.meas_full && P.stag[0] != 0.0) {
      const T o = one<T>();
      for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
        const int i = e % N, j = e / N;
        const double w = P.stag[i] * P.stag[j];
        const T gii = cvt<T>(G0[i + (size_t)i * N]), gjj = cvt<T>(G0[j + (size_t)j * N]);
        const T gij = cvt<T>(G0[e]), gji = cvt<T>(G0[j + (size_t)i * N]);
        const T del = i == j ? o : zero<T>();
        const double same = re((o - gii) * (o - gjj) + (del - gij) * gji) + re(conjg(gii * gjj + gij * (del - gji)));
        const double opp = re((o - gii) * conjg(gjj)) + re(conjg(gii) * (o - gjj));
        sf[4] += w * (same + opp);
        sf[6] += w * (same - opp);
      }
    }
  }
  ek = block_sum(ek, c.sm.red);
  eu = block_sum(eu, c.sm.red);
  ev = block_sum(ev, c.sm.red);
  const int nsf = (KIND == KDQ_TV || P.meas_full) ? 8 : 4;
  for (int q = 0; q < nsf; ++q) sf[q] = block_sum(sf[q], c.sm.red);
  const double n2 = (double)N * N;
  if constexpr (KIND == KDQ_TU) {
    acc[0] = -2.0 * P.Ht * ek;
    acc[1] = eu;
    for (int q = 0; q < 4; ++q) acc[2 + q] = sf[q] / n2;
    if (P.meas_full)
      for (int q = 0; q < 4; ++q) acc[6 + q] = sf[4 + q] / n2;
  } else if constexpr (KIND == KDQ_TV) {
    acc[0] = P.Ht * ek;
    acc[1] = ev;
    for (int q = 0; q < 8; ++q) acc[2 + q] = sf[q] * 4.0 / n2;
  } else {
    acc[0] = 2.0 * P.Ht * ek;
    acc[1] = P.U * eu;
    acc[2] = P.V * ev;
    for (int q = 0; q < 4; ++q) acc[3 + q] = sf[q] / n2;
    if (P.meas_full)
      for (int q = 0; q < 4; ++q) acc[7 + q] = sf[4 + q] / n2;
  }
  if (threadIdx.x == 0) {
    for (int q = 0; q < P.n_obs; ++q) c.ctl->obs_acc[q] += acc[q];
    c.ctl->obs_cnt += 1;
  }
  __syncthreads();
}

// ------------------------------------------------- measurement, fast form
// record == 2: the same estimator as `measure`, with the wrap of the G copy
// to Nt/2 and the HalfeK symmetrisation folded into two N x N factors,
//   G0 = L G R,  L = HalfeK W,  R = W^-1 HalfeKinv,
// W = B_half ... B_{t0+1} (t0 <= Nt/2) or B_{half+1}^-1 ... B_{t0}^-1 (t0 > Nt/2)
// with the current fields.  L and R are kept between measurements as a
// stack of slice factors, each with the fields it was built from; a new
// measurement pops the factors whose slice or fields no longer match and
// pushes the missing ones (one or two of each between consecutive measured
// slices), instead of re-wrapping |t0 - Nt/2| slices.

// X <- X B_lt (right = true) or B_lt X, with B the slice matrix of `fields`
// (inv: B^-1).  W is N x N scratch.
template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void mul_slice(Ctx<KIND, T, KT, TW, KW>& c, TW* X, TW* W, int lt, const uint8_t* fields, bool right, bool inv) {
  const SweepParams& P = c.P;
  const int N = P.Ns;
  if constexpr (KIND == KDQ_TV) {
    // B = V_1 ... V_z eK, V_j = UV D_j UV (2x2 blocks (lp, lm)); V_j^-1 blocks (rp, rm)
    auto rot = [&](int j) {
      tv_coeffs(c, lt, j, +1, fields);
      const TW* Q = inv ? c.sm.dinv : c.sm.dvec;
      const int nb = N / 2;
      for (int e = threadIdx.x; e < nb * N; e += blockDim.x) {
        const int i = e % nb, o = e / nb;
        const int x = P.bx[j * nb + i], y = P.by[j * nb + i];
        const TW qp = Q[2 * i], qm = Q[2 * i + 1];
        TW* px = right ? X + (size_t)x * N + o : X + x + (size_t)o * N;
        TW* py = right ? X + (size_t)y * N + o : X + y + (size_t)o * N;
        const TW vx = *px, vy = *py;
        *px = vx * qp + vy * qm;
        *py = vx * qm + vy * qp;
      }
      __syncthreads();
    };
    const bool k_first = right == inv;   // X eKinv ... / eK X ... come first
    if (k_first) {
      if (right) gemm_sq<MAXRM, TW>(N, N, N, X, N, c.eKinv, N, W, N);
      else gemm_sq<MAXRM, TW>(N, N, N, c.eK, N, X, N, W, N);
      for (int e = threadIdx.x; e < N * N; e += blockDim.x) X[e] = W[e];
      __syncthreads();
    }
    // right: X V_1 V_2 ... (B) or X ... V_2^-1 V_1^-1 (B^-1, after eKinv)
    // left:  V_1 V_2 ... V_z (eK X) applied innermost-first, or V_1^-1 first for B^-1
    const bool ascending = right ? !inv : inv;
    for (int q = 0; q < P.z; ++q) rot(ascending ? q : P.z - 1 - q);
    if (!k_first) {
      if (right) gemm_sq<MAXRM, TW>(N, N, N, X, N, c.eK, N, W, N);
      else gemm_sq<MAXRM, TW>(N, N, N, c.eKinv, N, X, N, W, N);
      for (int e = threadIdx.x; e < N * N; e += blockDim.x) X[e] = W[e];
      __syncthreads();
    }
  } else {
    slice_diag(c, lt, +1, fields);   // dvec = D, dinv = 1 ./ D
    const TW* d = inv ? c.sm.dinv : c.sm.dvec;
    if (right && !inv) {          // X D eK
      for (Walk w(N, N); w.ok(); w.next()) X[w.e] = X[w.e] * d[w.j];
      __syncthreads();
      kmul_right<MAXRM, false>(N, N, N, X, N, c.eK, kin_frag(c.P, KIN_EK, 1), N, W, N);
    } else if (right) {           // X eKinv D^-1
      kmul_right<MAXRM, false>(N, N, N, X, N, c.eKinv, kin_frag(c.P, KIN_EKINV, 1), N, W, N, (const TW*)nullptr, d);
    } else if (!inv) {            // D eK X
      kmul_left<MAXRM, false>(N, N, N, c.eK, kin_frag(c.P, KIN_EK, 0), N, X, N, W, N, d, (const TW*)nullptr);
    } else {                      // eKinv D^-1 X
      for (Walk w(N, N); w.ok(); w.next()) X[w.e] = d[w.i] * X[w.e];
      __syncthreads();
      kmul_left<MAXRM, false>(N, N, N, c.eKinv, kin_frag(c.P, KIN_EKINV, 0), N, X, N, W, N);
    }
    for (int e = threadIdx.x; e < N * N; e += blockDim.x) X[e] = W[e];
    __syncthreads();
  }
}

template <int MAXRM, int KIND, class T, class KT, class TW, class KW>
__device__ void measure_fast(Ctx<KIND, T, KT, TW, KW>& c, int t0) {
  const SweepParams& P = c.P;
  keep_middle(c, t0);
  const int N = P.Ns, half = P.Nt / 2, nf = P.n_field;
  TW* L = static_cast<TW*>(P.Lm) + (size_t)c.chain * P.sz_NN;
  TW* R = static_cast<TW*>(P.Rm) + (size_t)c.chain * P.sz_NN;
  TW* W = c.W1;
  int* fslice = reinterpret_cast<int*>(P.mstack + (size_t)c.chain * P.mstack_stride);
  uint8_t* fsnap = P.mstack + (size_t)c.chain * P.mstack_stride + (size_t)P.mstack_max * sizeof(int);
  const bool below = 2 * t0 <= P.Nt;     // t0 <= Nt/2: factors B_half ... B_{t0+1}
  const int m = below ? half - t0 : t0 - half;
  auto target = [&](int q) { return below ? half - q : half + 1 + q; };   // slice of factor q
  auto orient = [&](int q) { return below ? +1 : -1; };
  const int n = c.ctl->meas_n;
  // slices carry their orientation in the sign of fslice
  __shared__ int match;
  int k = 0;
  for (; k < n && k < m; ++k) {
    if (threadIdx.x == 0) match = fslice[k] == orient(k) * target(k);
    __syncthreads();
    const uint8_t* cur = c.s + (size_t)(target(k) - 1) * nf;
    const uint8_t* snap = fsnap + (size_t)k * nf;
    int diff = 0;
    for (int i = threadIdx.x; i < nf; i += blockDim.x) diff |= cur[i] != snap[i];
    diff = __syncthreads_or(diff);
    if (!match || diff) break;
  }
  if (k == 0) {
    for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
      L[e] = cvt<TW>(c.HalfeK[e]);
      R[e] = cvt<TW>(c.HalfeKinv[e]);
    }
    __syncthreads();
  } else {
    for (int q = n - 1; q >= k; --q) {   // pop: undo factor q
      const int sl = fslice[q] > 0 ? fslice[q] : -fslice[q];
      const bool is_B = fslice[q] > 0;
      const uint8_t* snap = fsnap + (size_t)q * nf;
      mul_slice<MAXRM>(c, L, W, sl, snap, true, is_B);    // L <- L F^-1
      mul_slice<MAXRM>(c, R, W, sl, snap, false, !is_B);  // R <- F R
    }
  }
  for (int q = k; q < m; ++q) {          // push factor q with the current fields
    const int sl = target(q);
    const bool is_B = orient(q) > 0;
    const uint8_t* cur = c.s + (size_t)(sl - 1) * nf;
    mul_slice<MAXRM>(c, L, W, sl, cur, true, !is_B);     // L <- L F
    mul_slice<MAXRM>(c, R, W, sl, cur, false, is_B);     // R <- F^-1 R
    uint8_t* snap = fsnap + (size_t)q * nf;
    for (int i = threadIdx.x; i < nf; i += blockDim.x) snap[i] = cur[i];
    if (threadIdx.x == 0) fslice[q] = orient(q) * sl;
  }
  if (threadIdx.x == 0) c.ctl->meas_n = m;
  __syncthreads();
  gemm_sq<MAXRM, TW>(N, N, N, L, N, c.G, N, W, N);
  gemm_sq<MAXRM, TW>(N, N, N, W, N, R, N, c.W2, N);
  observables(c, c.W2);
}

// ------------------------------------------------------------------ kernel
template <int KIND, class T, class KT, int MAXRM, bool MIXED, class C>
__device__ __forceinline__ void sweep_block(C& c, const SweepParams& P, int mode, int k);

// mode KDQ_MODE_INIT: block k of the initial left chain (and G at k == 1);
// KDQ_MODE_FWD: forward slices node(k)+1 .. node(k+1), then the node;
// KDQ_MODE_BWD: backward slices node(k+1) .. node(k)+1, then the node;
// KDQ_MODE_SWEEP: all forward then all backward blocks of one sweep.
// MIXED selects the mixed precision (see the header of this file).
template <int KIND, class T, class KT, int MAXRM, bool MIXED>
__global__ void __launch_bounds__(KDQ_THREADS, 2) k_block(const SweepParams P, int mode, int k) {
  using TW = std::conditional_t<MIXED, typename low_t<T>::type, T>;
  using KW = std::conditional_t<MIXED, typename low_t<KT>::type, KT>;
  using TS = typename Ctx<KIND, T, KT, TW, KW>::TS;
  extern __shared__ double dyn_d[];
  __shared__ Smem<TW> sm;
  const int chain = blockIdx.x;
  const int N = P.Ns;
  PhaseClock clk;
  clk.start(P.phase ? P.phase + (size_t)chain * 8 : nullptr);
  const size_t cNN = (size_t)chain * P.sz_NN;
  const size_t cNn = (size_t)chain * P.sz_Nn;
  Ctx<KIND, T, KT, TW, KW> c{P,
                             sm,
                             reinterpret_cast<uint8_t*>(dyn_d + P.n_field),
                             dyn_d,
                             chain,
                             P.ctl + chain,
                             static_cast<TW*>(P.G) + cNN,
                             static_cast<TW*>(P.W1) + cNN,
                             static_cast<TW*>(P.W2) + cNN,
                             static_cast<TW*>(P.Yw) + cNn,
                             static_cast<TW*>(P.Y2w) + cNn,
                             static_cast<TS*>(P.Y) + cNn,
                             static_cast<TS*>(P.Y2) + cNn,
                             static_cast<TS*>(P.Gd) + cNN,
                             static_cast<TS*>(P.Mss) + (size_t)chain * P.sz_nn,
                             static_cast<TS*>(P.X) + cNn,
                             P.piv + (size_t)chain * (N / 2),
                             P.s + (size_t)chain * P.Nt * P.n_field,
                             static_cast<const KW*>(P.eK),
                             static_cast<const KW*>(P.eKinv),
                             static_cast<const KW*>(P.HalfeK),
                             static_cast<const KW*>(P.HalfeKinv),
                             static_cast<const KT*>(P.K),
                             clk};
  if constexpr (KIND == KDQ_TU) {
    if (P.slmc_moves > 0 && mode != KDQ_MODE_INIT) {
      c.slmc = reinterpret_cast<unsigned char*>(dyn_d) + P.slmc_off;
      load_cnn_weights(*reinterpret_cast<CnnW*>(c.slmc), static_cast<const __nv_bfloat16*>(P.slmc_prm));
    }
  }
  if (mode == KDQ_MODE_INIT) {
    node_backward<MAXRM>(c, k, k == 1, false);
    return;
  }
  // KDQ_MODE_SWEEP: the whole sweep in one launch (a chain's blocks depend
  // only on that chain, so each CTA runs through them without waiting for
  // the others); one call site keeps the block body inlined once
  const int nb = mode == KDQ_MODE_SWEEP ? 2 * (P.NN - 1) : 1;
  for (int b = 0; b < nb; ++b) {
    int m = mode, kk = k;
    if (mode == KDQ_MODE_SWEEP) {
      m = b < P.NN - 1 ? KDQ_MODE_FWD : KDQ_MODE_BWD;
      kk = b < P.NN - 1 ? b + 1 : 2 * (P.NN - 1) - b;
    }
    sweep_block<KIND, T, KT, MAXRM, MIXED>(c, P, m, kk);
  }
}

// One stabilisation block of the sweep: forward slices node(k)+1 .. node(k+1)
// then the node, or backward slices node(k+1) .. node(k)+1 then the node.
template <int KIND, class T, class KT, int MAXRM, bool MIXED, class C>
__device__ __forceinline__ void sweep_block(C& c, const SweepParams& P, int mode, int k) {
  const int N = P.Ns;
  const int chain = c.chain;
  PhaseClock& clk = c.clk;
  using TW = std::conditional_t<MIXED, typename low_t<T>::type, T>;
  const int Θidx = P.NN / 2 + 1;
  const int lo = (int)P.nodes[k - 1], hi = (int)P.nodes[k];
  if (mode == KDQ_MODE_FWD) {
    // idx == k while these slices run (src/tU/phy_update.jl:53-98)
    const bool rec = P.record && (KIND == KDQ_TU ? (Θidx - k >= 0 && Θidx - k <= 1) : abs(k - Θidx) <= 1);
    for (int lt = lo + 1; lt <= hi; ++lt) {
      if constexpr (KIND == KDQ_TV) {
        gemm_sq<MAXRM, TW>(N, N, N, c.G, N, c.eKinv, N, c.W1, N);
        gemm_sq<MAXRM, TW>(N, N, N, c.eK, N, c.W1, N, c.G, N);
        for (int j = P.z - 1; j >= 0; --j) {
          tv_rotate(c, c.G, lt, j, +1);
          clk.lap(0);
          update_layer<MAXRM>(c, lt, j, true);
          clk.lap(1);
        }
      } else {
        wrap_fwd_kv<MAXRM>(c, c.G, c.W1, lt);
        clk.lap(0);
        update_layer<MAXRM>(c, lt, 0, true);
        clk.lap(1);
        if constexpr (KIND == KDQ_TU) {
          if (c.slmc) {
            slmc_moves<MAXRM>(c, lt, lt - 1);
            clk.lap(6);
          }
        }
      }
      if (rec) {
        if (P.record == 2) measure_fast<MAXRM>(c, lt);
        else measure<MAXRM>(c, lt);
        clk.lap(2);
      }
    }
    clk.lap(0);
    node_forward<MAXRM>(c, k);
  } else {
    // idx == k+1 while these slices run (src/tU/phy_update.jl:101-139)
    const int idx = k + 1;
    const bool rec = P.record && (KIND == KDQ_TU ? (idx - Θidx >= 0 && idx - Θidx <= 1) : abs(idx - Θidx) <= 1);
    for (int lt = hi; lt > lo; --lt) {
      if constexpr (KIND == KDQ_TV) {
        for (int j = 0; j < P.z; ++j) {
          update_layer<MAXRM>(c, lt, j, false);
          clk.lap(1);
          tv_rotate(c, c.G, lt, j, -1);
          clk.lap(0);
        }
        gemm_sq<MAXRM, TW>(N, N, N, c.eKinv, N, c.G, N, c.W1, N);
        gemm_sq<MAXRM, TW>(N, N, N, c.W1, N, c.eK, N, c.G, N);
        clk.lap(0);
        if (rec) {
          if (P.record == 2) measure_fast<MAXRM>(c, lt - 1);
          else measure<MAXRM>(c, lt - 1);
          clk.lap(2);
        }
      } else {
        update_layer<MAXRM>(c, lt, 0, false);
        clk.lap(1);
        if constexpr (KIND == KDQ_TU) {
          if (c.slmc) {
            slmc_moves<MAXRM>(c, lt, 2 * P.Nt - lt);
            clk.lap(6);
          }
        }
        if (rec) {
          if (P.record == 2) measure_fast<MAXRM>(c, lt);
          else measure<MAXRM>(c, lt);
          clk.lap(2);
        }
        wrap_bwd_kv<MAXRM>(c, c.G, c.W1, lt);
        clk.lap(0);
      }
    }
    clk.lap(0);
    node_backward<MAXRM>(c, k, true, true);
    if (k == 1 && threadIdx.x == 0) {
      ChainCtl* ctl = c.ctl;
      if (P.record) {
        if (ctl->obs_slot < P.obs_cap) {
          double* row = P.obs + ((size_t)chain * P.obs_cap + ctl->obs_slot) * P.n_obs;
          for (int q = 0; q < P.n_obs; ++q) row[q] = ctl->obs_acc[q] / ctl->obs_cnt;
        }
        ctl->obs_slot += 1;
        for (int q = 0; q < KDQ_MAX_OBS; ++q) ctl->obs_acc[q] = 0.0;
        ctl->obs_cnt = 0;
      }
      ctl->sweep += 1;
    }
  }
}

}  // namespace kdq
