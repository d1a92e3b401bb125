// Coupled incremental SCEE sweep (t-U): ctrl_SCEEicr, src/tU/SCEE.jl:1-324.
//
// One CTA per replica pair (chains 2p and 2p+1 of the handle), one launch
// per stabilisation block, like the plain sweep.  Each replica keeps four
// Green's functions (G4Buffer_, src/public/Buffer.jl:22-31): Gt = G(tau,tau)
// in the chain's G buffer, G0 = G(tau0,tau0) at the middle node, Gt0 =
// G(tau,tau0) and G0t = G(tau0,tau); the pair keeps the inverse Grover
// matrices of regions A and B and |det g_A|^2, |det g_B|^2.  A proposal of
// replica r at site i is accepted with
//   |1 + Delta (1 - Gt_ii)|^2 gamma'/gamma |Tau_A|^(2 lambda) |Tau_B|^(2 (1 - lambda))
// where Tau = 1 + b a is the rank-1 change of the Grover determinant
// (get_abTau1!/get_abTau2!, src/public/Gupdate.jl:91-132); on acceptance the
// inverse Grover matrices take a rank-1 update (GMupdate!, :45-58) and the
// replica's four Green's functions the rank-1 updates of G4update! (:23-37).
// At every node the block products of both replicas are rebuilt and the four
// Green's functions recomputed from the stabilised chains (G4!, :159-212).
#pragma once
#include "kdq_sweep.cuh"

namespace kdq {

#define KDQ_SCEE_MAXR 96   // largest region (sites)

// bytes of the two tape slices at the start of the dynamic shared memory
__host__ __device__ inline size_t scee_tape_bytes(int N) { return ((size_t)N * 18 + 15) & ~size_t(15); }

template <class T>
struct SceeSmem {
  T a[2][KDQ_SCEE_MAXR];      // per region: a, b, y vectors of the rank-1 Grover update
  T b[2][KDQ_SCEE_MAXR];
  T y[2][KDQ_SCEE_MAXR];
  T v[KDQ_SCEE_MAXR];
  T part[8][KDQ_SCEE_MAXR];   // per-warp partial sums of the vector-matrix products
  T tau[2];
  T rr;
  int acc;
  int bad;
};

// the same for the rank-2 (bond) updates of the t-V and t-UV sweeps
template <class T>
struct SceeSmem2 {
  T a[2][2][KDQ_SCEE_MAXR];   // [region][column of S][site]
  T b[2][2][KDQ_SCEE_MAXR];   // [region][row of S][site]
  T y[2][2][KDQ_SCEE_MAXR];
  T v[2][KDQ_SCEE_MAXR];
  T w[2][KDQ_SCEE_MAXR];
  T part[8][KDQ_SCEE_MAXR];
  T g4[8][KDQ_MAX_NS];        // staged columns and rows of the rank-2 Green's-function update
  T tau[2][4];
  T rr[4];
  int acc;
};

// out[j] = sum_l v[l] M(l, j), j < n (M given as an accessor); all threads
template <class T, class MF>
__device__ void vecmat(int n, const T* v, MF M, T* out, T (*part)[KDQ_SCEE_MAXR]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int j = j0 + lane;
    T s = zero<T>();
    if (j < n)
      for (int l = warp; l < n; l += nw) madd(s, v[l], M(l, j));
    if (j < n) part[warp][j] = s;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    T s = zero<T>();
    for (int w = 0; w < nw; ++w) s = s + part[w][j];
    out[j] = s;
  }
  __syncthreads();
}

// out[l] = sum_j M(l, j) v[j]
template <class T, class MF>
__device__ void matvec(int n, MF M, const T* v, T* out, T (*part)[KDQ_SCEE_MAXR]) {
  vecmat<T>(n, v, [&](int j, int l) { return M(l, j); }, out, part);
}

// per-chain SCEE buffers
template <class T>
struct SceeChain {
  T* G0;
  T* Gt0;
  T* G0t;
  T* BMs;   // (NN-1) blocks, block k (1-based) at (k-1) * N*N
  T* BMi;
};

template <class T>
__device__ inline SceeChain<T> scee_chain(const SweepParams& P, int chain) {
  const size_t NN2 = (size_t)P.Ns * P.Ns;
  SceeChain<T> s;
  s.G0 = static_cast<T*>(P.scee_G0) + (size_t)chain * NN2;
  s.Gt0 = static_cast<T*>(P.scee_Gt0) + (size_t)chain * NN2;
  s.G0t = static_cast<T*>(P.scee_G0t) + (size_t)chain * NN2;
  s.BMs = static_cast<T*>(P.scee_BMs) + (size_t)chain * (P.NN - 1) * NN2;
  s.BMi = static_cast<T*>(P.scee_BMi) + (size_t)chain * (P.NN - 1) * NN2;
  return s;
}

// copy / fill helpers (whole CTA)
template <class T>
__device__ void mcopy(int n, const T* src, T* dst) {
  for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = src[e];
  __syncthreads();
}

// One-sided bond rotations of direction j of slice lt on an N x N matrix
// (WrapV! "L" and "R", src/tV/GreenMatrix.jl:99-119): tv_left applies V_j
// (sign +1) or V_j^-1 (sign -1) from the left, tv_right V_j^-1 (sign +1) or
// V_j (sign -1) from the right, each as the 2x2 blocks on the bond's rows or
// columns.
template <int KIND, class T, class KT>
__device__ void tv_left(Ctx<KIND, T, KT, T, KT>& c, T* M, int lt, int j, int sign) {
  const SweepParams& P = c.P;
  const int N = P.Ns, nb = N / 2;
  tv_coeffs(c, lt, j, sign);
  const T* L = c.sm.dvec;
  const int* bx = P.bx + (size_t)j * nb;
  const int* by = P.by + (size_t)j * nb;
  for (Walk w(nb, N); w.ok(); w.next()) {
    const int x = bx[w.i], y = by[w.i];
    const T lp = L[2 * w.i], lm = L[2 * w.i + 1];
    const T gx = M[x + (size_t)w.j * N], gy = M[y + (size_t)w.j * N];
    M[x + (size_t)w.j * N] = lp * gx + lm * gy;
    M[y + (size_t)w.j * N] = lm * gx + lp * gy;
  }
  __syncthreads();
}

template <int KIND, class T, class KT>
__device__ void tv_right(Ctx<KIND, T, KT, T, KT>& c, T* M, int lt, int j, int sign) {
  const SweepParams& P = c.P;
  const int N = P.Ns, nb = N / 2;
  tv_coeffs(c, lt, j, sign);
  const T* R = c.sm.dinv;
  const int* bx = P.bx + (size_t)j * nb;
  const int* by = P.by + (size_t)j * nb;
  for (Walk w(N, nb); w.ok(); w.next()) {
    const int xp = bx[w.j], yp = by[w.j];
    const T rp = R[2 * w.j], rm = R[2 * w.j + 1];
    const T a = M[w.i + (size_t)xp * N], b = M[w.i + (size_t)yp * N];
    M[w.i + (size_t)xp * N] = a * rp + b * rm;
    M[w.i + (size_t)yp * N] = a * rm + b * rp;
  }
  __syncthreads();
}

// Block product of block k and its inverse (BM_F!, BMinv_F!,
// src/tU/GreenMatrix.jl:10-47): BM = prod D eK, BMinv = prod eKinv D^-1.
template <int MAXRM, int KIND, class T, class KT>
__device__ __noinline__ void scee_block_mats(Ctx<KIND, T, KT, T, KT>& c, int k, T* BM, T* BMi) {
  const SweepParams& P = c.P;
  const int N = P.Ns;
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
    BM[e] = (e % N == e / N) ? one<T>() : zero<T>();
    BMi[e] = BM[e];
  }
  __syncthreads();
  for (int lt = (int)P.nodes[k - 1] + 1; lt <= (int)P.nodes[k]; ++lt) {
    if constexpr (KIND == KDQ_TV) {   // B = V_1 .. V_z eK, B^-1 = eKinv V_z^-1 .. V_1^-1
      gemm_sq<MAXRM, T>(N, N, N, c.eK, N, BM, N, c.W1, N);
      mcopy(N * N, c.W1, BM);
      gemm_sq<MAXRM, T>(N, N, N, BMi, N, c.eKinv, N, c.W1, N);
      mcopy(N * N, c.W1, BMi);
      for (int j = P.z - 1; j >= 0; --j) {
        tv_left(c, BM, lt, j, +1);
        tv_right(c, BMi, lt, j, +1);
      }
    } else {
      slice_diag(c, lt, +1);
      gemm_sq<MAXRM, T>(N, N, N, c.eK, N, BM, N, c.W1, N, c.sm.dvec, (const T*)nullptr);
      mcopy(N * N, c.W1, BM);
      gemm_sq<MAXRM, T>(N, N, N, BMi, N, c.eKinv, N, c.W1, N, (const T*)nullptr, c.sm.dinv);
      mcopy(N * N, c.W1, BMi);
    }
  }
}

// BR[i] = orth_cols(BMs[i-1] BR[i-1])
template <int MAXRM, int KIND, class T, class KT>
__device__ __noinline__ void scee_br(Ctx<KIND, T, KT, T, KT>& c, const SceeChain<T>& q, int i) {
  const int N = c.P.Ns, ns = N / 2;
  const size_t fs = (size_t)N * ns;
  const SweepParams& P = c.P;
  T* BR = P.BRs<T>(c.chain);
  gemm_thin<MAXRM, T>(N, ns, N, q.BMs + (size_t)(i - 2) * N * N, N, BR + (size_t)(i - 2) * fs, N, c.Y, N);
  householder_q(N, ns, c.Y, BR + (size_t)(i - 1) * fs, c.sm.wn, c.sm.red);
}

// BL[i] = orth_rows(BL[i+1] BMs[i])
template <int MAXRM, int KIND, class T, class KT>
__device__ __noinline__ void scee_bl(Ctx<KIND, T, KT, T, KT>& c, const SceeChain<T>& q, int i) {
  const int N = c.P.Ns, ns = N / 2;
  const size_t fs = (size_t)N * ns;
  const SweepParams& P = c.P;
  T* BL = P.BLs<T>(c.chain);
  gemm_thin<MAXRM, T>(ns, N, N, BL + (size_t)i * fs, ns, q.BMs + (size_t)(i - 1) * N * N, N, c.Y2, ns);
  for (size_t e = threadIdx.x; e < fs; e += blockDim.x) {
    const int r = e % ns, col = e / ns;
    c.Y[col + (size_t)r * N] = conjg(c.Y2[e]);
  }
  __syncthreads();
  householder_q(N, ns, c.Y, c.X, c.sm.wn, c.sm.red);
  T* dst = BL + (size_t)(i - 1) * fs;
  for (size_t e = threadIdx.x; e < fs; e += blockDim.x) {
    const int r = e % ns, col = e / ns;
    dst[e] = conjg(c.X[col + (size_t)r * N]);
  }
  __syncthreads();
}

// out = I - BR (BL BR)^-1 BL at node i (get_G!, src/public/Gupdate.jl:139-157)
template <int MAXRM, int KIND, class T, class KT>
__device__ __noinline__ void scee_green(Ctx<KIND, T, KT, T, KT>& c, int i, T* out) {
  const int N = c.P.Ns, ns = N / 2;
  const size_t fs = (size_t)N * ns;
  const SweepParams& P = c.P;
  const T* BL = P.BLs<T>(c.chain) + (size_t)(i - 1) * fs;
  const T* BR = P.BRs<T>(c.chain) + (size_t)(i - 1) * fs;
  __shared__ int bad;
  __shared__ T fcol[KDQ_MAX_NS / 2];
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  gemm_thin<MAXRM, T>(ns, ns, N, BL, ns, BR, N, c.Mss, ns);
  gj_inverse(ns, c.Mss, fcol, c.piv, &bad);
  gemm_thin<MAXRM, T>(ns, N, ns, c.Mss, ns, BL, ns, c.X, ns);
  gemm_sq<MAXRM, T>(N, N, ns, BR, N, c.X, ns, out, N);
  for (Walk w(N, N); w.ok(); w.next()) {
    T g = zero<T>() - out[w.e];
    if (w.i == w.j) g = g + one<T>();
    out[w.e] = g;
  }
  if (threadIdx.x == 0 && bad) atomicOr(&c.ctl->err, KDQ_FLAG_SINGULAR);
  __syncthreads();
}

// G4!: the four Green's functions of one replica at node idx
template <int MAXRM, int KIND, class T, class KT>
__device__ __noinline__ void scee_g4(Ctx<KIND, T, KT, T, KT>& c, const SceeChain<T>& q, int idx, bool fwd) {
  const SweepParams& P = c.P;
  const int N = P.Ns, NN2 = N * N, Th = P.NN / 2 + 1;
  T* Gt = c.G;
  scee_green<MAXRM>(c, idx, Gt);
  if (idx == Th) {
    for (Walk w(N, N); w.ok(); w.next()) {
      const T g = Gt[w.e];
      const T gm = w.i == w.j ? g - one<T>() : g;
      q.G0[w.e] = g;
      q.Gt0[w.e] = fwd ? g : gm;
      q.G0t[w.e] = fwd ? gm : g;
    }
    __syncthreads();
    return;
  }
  scee_green<MAXRM>(c, Th, q.G0);
  for (Walk w(N, N); w.ok(); w.next()) {
    const T v = w.i == w.j ? one<T>() : zero<T>();
    q.Gt0[w.e] = v;
    q.G0t[w.e] = v;
  }
  __syncthreads();
  // the product runs from the node nearer tau = 0 to the farther one:
  // idx < Th: G0t <- BM_j G_j G0t, Gt0 <- Gt0 (I - G_j) BMinv_j, then Gt0 = -Gt0
  // idx > Th: Gt0 <- BM_j G_j Gt0, G0t <- G0t (I - G_j) BMinv_j, then G0t = -G0t
  T* L = idx < Th ? q.G0t : q.Gt0;   // left-multiplied chain
  T* R = idx < Th ? q.Gt0 : q.G0t;   // right-multiplied chain
  const int j0 = idx < Th ? idx : Th, j1 = idx < Th ? Th : idx;
  for (int j = j0; j < j1; ++j) {
    const T* Gj;
    if (j == idx) Gj = Gt;
    else if (j == Th) Gj = q.G0;
    else {
      scee_green<MAXRM>(c, j, c.W2);
      Gj = c.W2;
    }
    gemm_sq<MAXRM, T>(N, N, N, Gj, N, L, N, c.W1, N);
    gemm_sq<MAXRM, T>(N, N, N, q.BMs + (size_t)(j - 1) * NN2, N, c.W1, N, L, N);
    gemm_sq<MAXRM, T>(N, N, N, R, N, Gj, N, c.W1, N);
    for (int e = threadIdx.x; e < NN2; e += blockDim.x) c.W1[e] = R[e] - c.W1[e];
    __syncthreads();
    gemm_sq<MAXRM, T>(N, N, N, c.W1, N, q.BMi + (size_t)(j - 1) * NN2, N, R, N);
  }
  for (int e = threadIdx.x; e < NN2; e += blockDim.x) R[e] = zero<T>() - R[e];
  __syncthreads();
}

// Grover matrix g = 2 a b - a - b + I of the replicas' G0 on a region; its
// inverse into inv and |det g|^2 (returned to thread 0)
template <int MAXRM, int KIND, class T, class KT>
__device__ __noinline__ double scee_grover(Ctx<KIND, T, KT, T, KT>& c, const T* G0a, const T* G0b, const int* idx, int n,
                              T* inv, T* wa, T* wb) {
  const int N = c.P.Ns;
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    const int i = e % n, j = e / n;
    wa[e] = G0a[idx[i] + (size_t)idx[j] * N];
    wb[e] = G0b[idx[i] + (size_t)idx[j] * N];
  }
  __syncthreads();
  gemm_sq<MAXRM, T>(n, n, n, wa, n, wb, n, inv, n);
  for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
    T g = 2.0 * inv[e] - wa[e] - wb[e];
    if (e % n == e / n) g = g + one<T>();
    inv[e] = g;
  }
  __syncthreads();
  __shared__ int bad;
  __shared__ T fcol[KDQ_SCEE_MAXR];
  __shared__ double lg;
  __shared__ cd ph;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  gj_inverse(n, inv, fcol, c.piv, &bad, &lg, &ph);
  if (threadIdx.x == 0 && bad) atomicOr(&c.ctl->err, KDQ_FLAG_SINGULAR);
  if constexpr (KIND == KDQ_TV) return ph.x * exp(lg);   // det g itself (src/tV/SCEE.jl:437)
  return exp(2.0 * lg);                                   // |det g|^2 (src/tU/SCEE.jl:268)
}

// Disorder-operator matrix X = e^{i alpha} I + (1 - e^{i alpha}) G0[R,R] of a
// region (get_ABX!, src/tU/disorder_operate.jl:202-224): inverse into inv,
// |det X|^2 returned
template <int MAXRM, int KIND, class T, class KT>
__device__ __noinline__ double scee_xmat(Ctx<KIND, T, KT, T, KT>& c, const T* G0, const int* idx, int n, T* inv) {
  const int N = c.P.Ns;
  double sn, cs;
  sincos(c.P.scee_alpha, &sn, &cs);
  const T e = cvt<T>(cd{cs, sn});
  const T om = one<T>() - e;
  for (int q = threadIdx.x; q < n * n; q += blockDim.x) {
    const int i = q % n, j = q / n;
    T x = om * G0[idx[i] + (size_t)idx[j] * N];
    if (i == j) x = x + e;
    inv[q] = x;
  }
  __syncthreads();
  __shared__ int bad;
  __shared__ T fcol[KDQ_SCEE_MAXR];
  __shared__ double lg;
  __shared__ cd ph;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  gj_inverse(n, inv, fcol, c.piv, &bad, &lg, &ph);
  if (threadIdx.x == 0 && bad) atomicOr(&c.ctl->err, KDQ_FLAG_SINGULAR);
  return exp(2.0 * lg);
}

// get_ABGM! (get_ABX! for the disorder operator): four Green's functions of
// the replicas and the inverses of both region matrices
template <int MAXRM, int KIND, class T, class KT>
__device__ __noinline__ void scee_abgm(Ctx<KIND, T, KT, T, KT>* c, const SceeChain<T>* q, int idx, bool fwd, int pair) {
  const SweepParams& P = c[0].P;
  scee_g4<MAXRM>(c[0], q[0], idx, fwd);
  if (!P.scee_dop) scee_g4<MAXRM>(c[1], q[1], idx, fwd);
  const size_t rs = (size_t)P.scee_nmax * P.scee_nmax;
  T* invA = static_cast<T*>(P.scee_inv) + (size_t)pair * 2 * rs;
  T* invB = invA + rs;
  double dA = 0.0, dB = 0.0;
  if (P.scee_dop) {
    if constexpr (KIND == KDQ_TU) {
      dA = scee_xmat<MAXRM>(c[0], q[0].G0, P.scee_idxA, P.scee_nA, invA);
      dB = scee_xmat<MAXRM>(c[0], q[0].G0, P.scee_idxB, P.scee_nB, invB);
    }
  } else {
    dA = scee_grover<MAXRM>(c[0], q[0].G0, q[1].G0, P.scee_idxA, P.scee_nA, invA, c[0].W1, c[0].W2);
    dB = scee_grover<MAXRM>(c[0], q[0].G0, q[1].G0, P.scee_idxB, P.scee_nB, invB, c[0].W1, c[0].W2);
  }
  if (threadIdx.x == 0) {
    P.scee_det[(size_t)pair * 4 + 0] = dA;
    P.scee_det[(size_t)pair * 4 + 1] = dB;
  }
  __syncthreads();
}

// WrapKV! "L", "B", "R" of one replica (src/tU/GreenMatrix.jl:56-86; the
// backward "R" uses cis(+alpha eta) as the reference's in-place inversion of
// its diagonal in the preceding "B" call leaves it)
template <int MAXRM, int KIND, class T, class KT>
__device__ void scee_wrap(Ctx<KIND, T, KT, T, KT>& c, const SceeChain<T>& q, int lt, bool fwd) {
  const int N = c.P.Ns, NN2 = N * N;
  slice_diag(c, lt, +1);
  const T* d = c.sm.dvec;
  const T* di = c.sm.dinv;
  if (fwd) {
    gemm_sq<MAXRM, T>(N, N, N, c.eK, N, q.Gt0, N, c.W1, N, d, (const T*)nullptr);
    mcopy(NN2, c.W1, q.Gt0);
    gemm_sq<MAXRM, T>(N, N, N, c.eK, N, c.G, N, c.W1, N);
    gemm_sq<MAXRM, T>(N, N, N, c.W1, N, c.eKinv, N, c.G, N, d, di);
    gemm_sq<MAXRM, T>(N, N, N, q.G0t, N, c.eKinv, N, c.W1, N, (const T*)nullptr, di);
    mcopy(NN2, c.W1, q.G0t);
  } else {
    for (Walk w(N, N); w.ok(); w.next()) {
      q.Gt0[w.e] = q.Gt0[w.e] * di[w.i];
      c.G[w.e] = c.G[w.e] * (di[w.i] * d[w.j]);
      q.G0t[w.e] = q.G0t[w.e] * d[w.j];
    }
    __syncthreads();
    gemm_sq<MAXRM, T>(N, N, N, c.eKinv, N, q.Gt0, N, c.W1, N);
    mcopy(NN2, c.W1, q.Gt0);
    gemm_sq<MAXRM, T>(N, N, N, c.eKinv, N, c.G, N, c.W1, N);
    gemm_sq<MAXRM, T>(N, N, N, c.W1, N, c.eK, N, c.G, N);
    gemm_sq<MAXRM, T>(N, N, N, q.G0t, N, c.eK, N, c.W1, N);
    mcopy(NN2, c.W1, q.G0t);
  }
}

// One proposal of replica r (0 or 1) at site i of slice lt (UpdateSCEELayer!,
// src/tU/SCEE.jl:278-324); co / qo: the other replica.
template <int MAXRM, int KIND, class T, class KT>
__device__ void scee_propose(Ctx<KIND, T, KT, T, KT>& c, const SceeChain<T>& q, const SceeChain<T>& qo, int r,
                             int lt, int i, int kk, double u, long long logpos, SceeSmem<T>& ss, int pair) {
  const SweepParams& P = c.P;
  const int N = P.Ns;
  const size_t rs = (size_t)P.scee_nmax * P.scee_nmax;
  T* inv[2] = {static_cast<T*>(P.scee_inv) + (size_t)pair * 2 * rs, nullptr};
  inv[1] = inv[0] + rs;
  const int* ridx[2] = {P.scee_idxA, P.scee_idxB};
  const int rn[2] = {P.scee_nA, P.scee_nB};
  uint8_t* sl = c.s + (size_t)(lt - 1) * N;
  const int sold = sl[i];
  const int sx = kk + (kk + 1 >= sold ? 2 : 1);
  __shared__ double p0;
  if (threadIdx.x == 0) {   // get_r!, src/tU/GreenMatrix.jl:49-54
    const T dlt = reinterpret_cast<const T*>(P.rtab)[(size_t)(lt - 1) * 16 + (sold - 1) * 4 + sx - 1];
    const T pc = one<T>() + dlt * (one<T>() - c.G[i + (size_t)i * N]);
    ss.rr = dlt / pc;
    p0 = abs2(pc) * P.gratio[(sold - 1) * 4 + sx - 1];
  }
  __syncthreads();
  const T rr = ss.rr;
  for (int g = 0; g < 2; ++g) {
    const int n = rn[g];
    const int* ix = ridx[g];
    const T* iv = inv[g];
    auto X = [&](int l, int j) {   // 2 G0_other[A,A] - I
      T x = 2.0 * qo.G0[ix[l] + (size_t)ix[j] * N];
      return l == j ? x - one<T>() : x;
    };
    if (P.scee_dop) {   // get_abTau! (DOPBuffer_): a = (1 - e^{i alpha}) G0t[R,i] r, b = Gt0[i,R] Xinv
      double sn, cs;
      sincos(P.scee_alpha, &sn, &cs);
      const T om = one<T>() - cvt<T>(cd{cs, sn});
      for (int l = threadIdx.x; l < n; l += blockDim.x) {
        ss.a[g][l] = om * (q.G0t[ix[l] + (size_t)i * N] * rr);
        ss.v[l] = q.Gt0[i + (size_t)ix[l] * N];
      }
      __syncthreads();
      vecmat<T>(n, ss.v, [&](int l, int j) { return iv[l + (size_t)j * n]; }, ss.b[g], ss.part);
    } else if (r == 0) {   // get_abTau1!: a = G0t[A,i] r, b = Gt0[i,A] X inv
      for (int l = threadIdx.x; l < n; l += blockDim.x) {
        ss.a[g][l] = q.G0t[ix[l] + (size_t)i * N] * rr;
        ss.v[l] = q.Gt0[i + (size_t)ix[l] * N];
      }
      __syncthreads();
      vecmat<T>(n, ss.v, X, ss.y[g], ss.part);
      vecmat<T>(n, ss.y[g], [&](int l, int j) { return iv[l + (size_t)j * n]; }, ss.b[g], ss.part);
    } else {        // get_abTau2!: a = X G0t[A,i], b = r Gt0[i,A] inv
      for (int l = threadIdx.x; l < n; l += blockDim.x) {
        ss.y[g][l] = q.G0t[ix[l] + (size_t)i * N];
        ss.v[l] = rr * q.Gt0[i + (size_t)ix[l] * N];
      }
      __syncthreads();
      matvec<T>(n, X, ss.y[g], ss.a[g], ss.part);
      vecmat<T>(n, ss.v, [&](int l, int j) { return iv[l + (size_t)j * n]; }, ss.b[g], ss.part);
    }
    // tau = 1 + b . a
    T t = zero<T>();
    for (int l = threadIdx.x; l < n; l += blockDim.x) madd(t, ss.b[g][l], ss.a[g][l]);
    t = warp_sum(t);
    if ((threadIdx.x & 31) == 0) ss.part[threadIdx.x >> 5][0] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
      T tt = one<T>();
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tt = tt + ss.part[w][0];
      ss.tau[g] = tt;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double dA = abs2(ss.tau[0]), dB = abs2(ss.tau[1]);
    const double p = p0 * (pow(dA, P.scee_lam) * pow(dB, 1.0 - P.scee_lam));
    int acc = u < p;
    if (!isfinite(p)) {
      acc = 0;
      atomicOr(&c.ctl->err, KDQ_FLAG_NAN);
    }
    ss.acc = acc;
    if (acc) {
      P.scee_det[(size_t)pair * 4 + 0] *= dA;
      P.scee_det[(size_t)pair * 4 + 1] *= dB;
    }
    if (P.acc_log && logpos < P.acc_log_cap) P.acc_log[(size_t)c.chain * P.acc_log_cap + logpos] = (uint8_t)acc;
    c.ctl->n_prop += 1;
    c.ctl->n_acc += acc;
  }
  __syncthreads();
  if (!ss.acc) return;
  // GMupdate!: inv <- inv - (inv a) (b / tau)
  for (int g = 0; g < 2; ++g) {
    const int n = rn[g];
    T* iv = inv[g];
    matvec<T>(n, [&](int l, int j) { return iv[l + (size_t)j * n]; }, ss.a[g], ss.y[g], ss.part);
    const T it = one<T>() / ss.tau[g];
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int l = e % n, j = e / n;
      iv[e] = iv[e] - ss.y[g][l] * (ss.b[g][j] * it);
    }
    __syncthreads();
  }
  // G4update!: z1 = r Gt0[i,:], z2 = E_i r - r Gt[i,:];
  // G0 += G0t[:,i] z1, Gt0 += Gt[:,i] z1, G0t -= G0t[:,i] z2, Gt -= Gt[:,i] z2
  T* c0t = c.sm.ucol[0];
  T* ct = c.sm.ucol[1];
  T* z1 = c.sm.wrow[0];
  T* z2 = c.sm.wrow[1];
  for (int b = threadIdx.x; b < N; b += blockDim.x) {
    c0t[b] = q.G0t[b + (size_t)i * N];
    ct[b] = c.G[b + (size_t)i * N];
    z1[b] = rr * q.Gt0[i + (size_t)b * N];
    T w = zero<T>() - rr * c.G[i + (size_t)b * N];
    if (b == i) w = w + rr;
    z2[b] = w;
  }
  __syncthreads();
  for (Walk w(N, N); w.ok(); w.next()) {
    const T a0 = c0t[w.i], a1 = ct[w.i], b1 = z1[w.j], b2 = z2[w.j];
    q.G0[w.e] = q.G0[w.e] + a0 * b1;
    q.Gt0[w.e] = q.Gt0[w.e] + a1 * b1;
    q.G0t[w.e] = q.G0t[w.e] - a0 * b2;
    c.G[w.e] = c.G[w.e] - a1 * b2;
  }
  if (threadIdx.x == 0) sl[i] = (uint8_t)sx;
  __syncthreads();
}

// the estimator (detg_A / detg_B)^(1/Nlambda) after every slice's updates
__device__ inline void scee_accumulate(const SweepParams& P, int pair) {
  if (threadIdx.x == 0) {
    double* dt = P.scee_det + (size_t)pair * 4;
    dt[2] += pow(dt[0] / dt[1], 1.0 / P.scee_nlam);
    dt[3] += 1.0;
  }
}

template <int MAXRM, int KIND, class T, class KT>
__device__ void scee_layer(Ctx<KIND, T, KT, T, KT>* c, const SceeChain<T>* q, int lt, bool fwd, SceeSmem<T>& ss,
                           int pair) {
  const SweepParams& P = c[0].P;
  const int N = P.Ns, Nt = P.Nt;
  const uint32_t qs = fwd ? (uint32_t)(lt - 1) * N : (uint32_t)(Nt + (Nt - lt)) * N;
  const bool two = !P.scee_dop;
  load_tape(c[0], qs, N);
  if (two) load_tape(c[1], qs, N);
  const long long lb0 = c[0].ctl->log_pos, lb1 = c[1].ctl->log_pos;
  for (int i = 0; i < N; ++i) {
    scee_propose<MAXRM>(c[0], q[0], q[1], 0, lt, i, c[0].tk[i], c[0].tu[i], lb0 + i, ss, pair);
    if (two) scee_propose<MAXRM>(c[1], q[1], q[0], 1, lt, i, c[1].tk[i], c[1].tu[i], lb1 + i, ss, pair);
  }
  if (threadIdx.x == 0) {
    c[0].ctl->log_pos += N;
    if (two) c[1].ctl->log_pos += N;
  }
  scee_accumulate(P, pair);
  finish_tape(c[0], N);
  if (two) finish_tape(c[1], N);
  __syncthreads();
}

// ------------------------------------------------------------------ t-V
// WrapK! (src/tV/SCEE.jl:509-517): Gt <- A Gt A^-1, Gt0 <- A Gt0, G0t <- G0t A^-1
// with A = eK (forward) or eKinv (backward)
template <int MAXRM, int KIND, class T, class KT>
__device__ void scee_wrapk(Ctx<KIND, T, KT, T, KT>& c, const SceeChain<T>& q, bool fwd) {
  const int N = c.P.Ns, NN2 = N * N;
  const KT* A = fwd ? c.eK : c.eKinv;
  const KT* Ai = fwd ? c.eKinv : c.eK;
  gemm_sq<MAXRM, T>(N, N, N, c.G, N, Ai, N, c.W1, N);
  gemm_sq<MAXRM, T>(N, N, N, A, N, c.W1, N, c.G, N);
  gemm_sq<MAXRM, T>(N, N, N, A, N, q.Gt0, N, c.W1, N);
  mcopy(NN2, c.W1, q.Gt0);
  gemm_sq<MAXRM, T>(N, N, N, q.G0t, N, Ai, N, c.W1, N);
  mcopy(NN2, c.W1, q.G0t);
}

// WrapV! "L", "B", "R" of direction j: V_j (forward) or V_j^-1 (backward)
template <int MAXRM, int KIND, class T, class KT>
__device__ void scee_wrapv(Ctx<KIND, T, KT, T, KT>& c, const SceeChain<T>& q, int lt, int j, bool fwd) {
  const int sign = fwd ? +1 : -1;
  tv_left(c, q.Gt0, lt, j, sign);
  tv_rotate(c, c.G, lt, j, sign);
  tv_right(c, q.G0t, lt, j, sign);
}

// One bond proposal of replica r at sites S = (x, y) (UpdateSCEELayer!,
// t-V src/tV/SCEE.jl:447-508, t-UV src/tUV/SCEE.jl:355-402): rank-2
// versions of get_abTau1!/get_abTau2!, GMupdate! and G4update!.  t-V weighs
// with det Tau (real), t-UV with |det Tau|^2; t-UV's local ratio is |det r|^2
// times the gamma ratio only (the reference's SCEE update leaves out the
// plain sweep's real-type factor).
template <int MAXRM, int KIND, class T, class KT>
__device__ void scee_propose2(Ctx<KIND, T, KT, T, KT>& c, const SceeChain<T>& q, const SceeChain<T>& qo, int r,
                              int lt, int x, int y, uint8_t* sf, int kk, double u, long long logpos,
                              SceeSmem2<T>& ss, int pair) {
  const SweepParams& P = c.P;
  const int N = P.Ns;
  const size_t rs = (size_t)P.scee_nmax * P.scee_nmax;
  T* inv[2] = {static_cast<T*>(P.scee_inv) + (size_t)pair * 2 * rs, nullptr};
  inv[1] = inv[0] + rs;
  const int* ridx[2] = {P.scee_idxA, P.scee_idxB};
  const int rn[2] = {P.scee_nA, P.scee_nB};
  const int S[2] = {x, y};
  const int sold = *sf;
  const int sx = kk + (kk + 1 >= sold ? 2 : 1);
  const T* G = c.G;
  __shared__ double p0;
  if (threadIdx.x == 0) {
    const T g00 = G[S[0] + (size_t)S[0] * N], g01 = G[S[0] + (size_t)S[1] * N];
    const T g10 = G[S[1] + (size_t)S[0] * N], g11 = G[S[1] + (size_t)S[1] * N];
    if constexpr (KIND == KDQ_TV) {   // get_r!, src/tV/GreenMatrix.jl:76-89
      const double h = 0.70710678118654752440;
      const double* t2 = P.rtab + ((size_t)(lt - 1) * 16 + (sold - 1) * 4 + sx - 1) * 2;
      const double q00 = -h * t2[0], q01 = -h * t2[1], q10 = -h * t2[0], q11 = h * t2[1];
      const double d00 = q00 * -h + q01 * -h, d01 = q00 * -h + q01 * h;
      const double d10 = q10 * -h + q11 * -h, d11 = q10 * -h + q11 * h;
      double a00 = d00 - (d00 * g00 + d01 * g10), a01 = d01 - (d00 * g01 + d01 * g11);
      double a10 = d10 - (d10 * g00 + d11 * g10), a11 = d11 - (d10 * g01 + d11 * g11);
      a00 += 1.0;
      a11 += 1.0;
      const double det = a00 * a11 - a01 * a10;
      p0 = det * P.gratio[(sold - 1) * 4 + sx - 1];
      const double rd = 1.0 / det;
      const double i00 = a11 * rd, i01 = -a01 * rd, i10 = -a10 * rd, i11 = a00 * rd;
      ss.rr[0] = i00 * d00 + i01 * d10;   // r = (I + Delta (I - G_SS))^-1 Delta, row-major 2x2
      ss.rr[1] = i00 * d01 + i01 * d11;
      ss.rr[2] = i10 * d00 + i11 * d10;
      ss.rr[3] = i10 * d01 + i11 * d11;
    } else {                          // get_r!, src/tUV/GreenMatrix.jl:73-89
      const T* t2 = reinterpret_cast<const T*>(P.rtab) + (size_t)((sold - 1) * 4 + sx - 1) * 2;
      T a00 = t2[0] - t2[0] * g00, a01 = zero<T>() - t2[0] * g01;
      T a10 = zero<T>() - t2[1] * g10, a11 = t2[1] - t2[1] * g11;
      a00 = a00 + one<T>();
      a11 = a11 + one<T>();
      const T det = a00 * a11 - a01 * a10;
      p0 = abs2(det) * P.gratio[(sold - 1) * 4 + sx - 1];
      const T rd = one<T>() / det;
      ss.rr[0] = (a11 * rd) * t2[0];
      ss.rr[1] = ((zero<T>() - a01) * rd) * t2[1];
      ss.rr[2] = ((zero<T>() - a10) * rd) * t2[0];
      ss.rr[3] = (a00 * rd) * t2[1];
    }
  }
  __syncthreads();
  const T r00 = ss.rr[0], r01 = ss.rr[1], r10 = ss.rr[2], r11 = ss.rr[3];
  for (int g = 0; g < 2; ++g) {
    const int n = rn[g];
    const int* ix = ridx[g];
    const T* iv = inv[g];
    auto X = [&](int l, int m) {   // 2 G0_other[A,A] - I
      const T xv = 2.0 * qo.G0[ix[l] + (size_t)ix[m] * N];
      return l == m ? xv - one<T>() : xv;
    };
    auto IV = [&](int l, int m) { return iv[l + (size_t)m * n]; };
    if (r == 0) {   // a = G0t[A,S] r, b = Gt0[S,A] X inv
      for (int l = threadIdx.x; l < n; l += blockDim.x) {
        const T g0 = q.G0t[ix[l] + (size_t)S[0] * N], g1 = q.G0t[ix[l] + (size_t)S[1] * N];
        ss.a[g][0][l] = g0 * r00 + g1 * r10;
        ss.a[g][1][l] = g0 * r01 + g1 * r11;
        ss.v[0][l] = q.Gt0[S[0] + (size_t)ix[l] * N];
        ss.v[1][l] = q.Gt0[S[1] + (size_t)ix[l] * N];
      }
      __syncthreads();
      for (int qr = 0; qr < 2; ++qr) {
        vecmat<T>(n, ss.v[qr], X, ss.y[g][qr], ss.part);
        vecmat<T>(n, ss.y[g][qr], IV, ss.b[g][qr], ss.part);
      }
    } else {        // a = X G0t[A,S], b = r Gt0[S,A] inv
      for (int l = threadIdx.x; l < n; l += blockDim.x) {
        ss.y[g][0][l] = q.G0t[ix[l] + (size_t)S[0] * N];
        ss.y[g][1][l] = q.G0t[ix[l] + (size_t)S[1] * N];
        const T t0 = q.Gt0[S[0] + (size_t)ix[l] * N], t1 = q.Gt0[S[1] + (size_t)ix[l] * N];
        ss.v[0][l] = r00 * t0 + r01 * t1;
        ss.v[1][l] = r10 * t0 + r11 * t1;
      }
      __syncthreads();
      for (int qc = 0; qc < 2; ++qc) {
        matvec<T>(n, X, ss.y[g][qc], ss.a[g][qc], ss.part);
        vecmat<T>(n, ss.v[qc], IV, ss.b[g][qc], ss.part);
      }
    }
    // Tau = I + b a (2 x 2, row-major)
    T t[4] = {zero<T>(), zero<T>(), zero<T>(), zero<T>()};
    for (int l = threadIdx.x; l < n; l += blockDim.x)
      for (int e = 0; e < 4; ++e) madd(t[e], ss.b[g][e >> 1][l], ss.a[g][e & 1][l]);
    for (int e = 0; e < 4; ++e) {
      t[e] = warp_sum(t[e]);
      if ((threadIdx.x & 31) == 0) ss.part[threadIdx.x >> 5][e] = t[e];
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int e = 0; e < 4; ++e) {
        T tt = (e == 0 || e == 3) ? one<T>() : zero<T>();
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tt = tt + ss.part[w][e];
        ss.tau[g][e] = tt;
      }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const T tA = ss.tau[0][0] * ss.tau[0][3] - ss.tau[0][1] * ss.tau[0][2];
    const T tB = ss.tau[1][0] * ss.tau[1][3] - ss.tau[1][1] * ss.tau[1][2];
    double dA, dB;
    if constexpr (KIND == KDQ_TV) {   // det Tau (src/tV/SCEE.jl:458-459)
      dA = re(tA);
      dB = re(tB);
    } else {                          // |det Tau|^2 (src/tUV/SCEE.jl:366-367)
      dA = abs2(tA);
      dB = abs2(tB);
    }
    const double p = p0 * (pow(dA, P.scee_lam) * pow(dB, 1.0 - P.scee_lam));
    int acc = u < p;
    if (isnan(p)) {
      acc = 0;
      atomicOr(&c.ctl->err, KDQ_FLAG_NAN);
    }
    ss.acc = acc;
    if (acc) {
      P.scee_det[(size_t)pair * 4 + 0] *= dA;
      P.scee_det[(size_t)pair * 4 + 1] *= dB;
    }
    if (P.acc_log && logpos < P.acc_log_cap) P.acc_log[(size_t)c.chain * P.acc_log_cap + logpos] = (uint8_t)acc;
    c.ctl->n_prop += 1;
    c.ctl->n_acc += acc;
  }
  __syncthreads();
  if (!ss.acc) return;
  // GMupdate!: inv <- inv - (inv a) Tau^-1 b
  for (int g = 0; g < 2; ++g) {
    const int n = rn[g];
    T* iv = inv[g];
    auto IV = [&](int l, int m) { return iv[l + (size_t)m * n]; };
    for (int qc = 0; qc < 2; ++qc) matvec<T>(n, IV, ss.a[g][qc], ss.y[g][qc], ss.part);
    const T* tg = ss.tau[g];
    const T td = one<T>() / (tg[0] * tg[3] - tg[1] * tg[2]);
    const T t00 = tg[3] * td, t01 = (zero<T>() - tg[1]) * td, t10 = (zero<T>() - tg[2]) * td, t11 = tg[0] * td;
    for (int m = threadIdx.x; m < n; m += blockDim.x) {
      const T b0 = ss.b[g][0][m], b1 = ss.b[g][1][m];
      ss.w[0][m] = t00 * b0 + t01 * b1;
      ss.w[1][m] = t10 * b0 + t11 * b1;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int l = e % n, m = e / n;
      iv[e] = iv[e] - (ss.y[g][0][l] * ss.w[0][m] + ss.y[g][1][l] * ss.w[1][m]);
    }
    __syncthreads();
  }
  // G4update!: z1 = r Gt0[S,:], z2 = E_S r - r Gt[S,:]
  T* c0t0 = ss.g4[0];
  T* c0t1 = ss.g4[1];
  T* ct0 = ss.g4[2];
  T* ct1 = ss.g4[3];
  T* z10 = ss.g4[4];
  T* z11 = ss.g4[5];
  T* z20 = ss.g4[6];
  T* z21 = ss.g4[7];
  for (int b = threadIdx.x; b < N; b += blockDim.x) {
    c0t0[b] = q.G0t[b + (size_t)S[0] * N];
    c0t1[b] = q.G0t[b + (size_t)S[1] * N];
    ct0[b] = G[b + (size_t)S[0] * N];
    ct1[b] = G[b + (size_t)S[1] * N];
    const T t0 = q.Gt0[S[0] + (size_t)b * N], t1 = q.Gt0[S[1] + (size_t)b * N];
    z10[b] = r00 * t0 + r01 * t1;
    z11[b] = r10 * t0 + r11 * t1;
    const T g0 = G[S[0] + (size_t)b * N], g1 = G[S[1] + (size_t)b * N];
    T w0 = zero<T>() - (r00 * g0 + r01 * g1), w1 = zero<T>() - (r10 * g0 + r11 * g1);
    if (b == S[0]) { w0 = w0 + r00; w1 = w1 + r10; }
    if (b == S[1]) { w0 = w0 + r01; w1 = w1 + r11; }
    z20[b] = w0;
    z21[b] = w1;
  }
  __syncthreads();
  for (Walk w(N, N); w.ok(); w.next()) {
    const T a0 = c0t0[w.i], a1 = c0t1[w.i], e0 = ct0[w.i], e1 = ct1[w.i];
    const T y0 = z10[w.j], y1 = z11[w.j], x0 = z20[w.j], x1 = z21[w.j];
    q.G0[w.e] = q.G0[w.e] + (a0 * y0 + a1 * y1);
    q.Gt0[w.e] = q.Gt0[w.e] + (e0 * y0 + e1 * y1);
    q.G0t[w.e] = q.G0t[w.e] - (a0 * x0 + a1 * x1);
    c.G[w.e] = c.G[w.e] - (e0 * x0 + e1 * x1);
  }
  if (threadIdx.x == 0) *sf = (uint8_t)sx;
  __syncthreads();
}

// The bonds of direction j of slice lt, both replicas alternating per bond
template <int MAXRM, int KIND, class T, class KT>
__device__ void scee_layer_tv(Ctx<KIND, T, KT, T, KT>* c, const SceeChain<T>* q, int lt, int j, bool fwd,
                              SceeSmem2<T>& ss, int pair) {
  const SweepParams& P = c[0].P;
  const int nb = P.Ns / 2, Nt = P.Nt, pf = P.n_field;
  const uint32_t qs = fwd ? (uint32_t)(lt - 1) * pf : (uint32_t)(Nt + (Nt - lt)) * pf;
  const int off = (fwd ? (P.z - 1 - j) : j) * nb;
  load_tape(c[0], qs + off, nb);
  load_tape(c[1], qs + off, nb);
  const long long lb0 = c[0].ctl->log_pos, lb1 = c[1].ctl->log_pos;
  for (int i = 0; i < nb; ++i) {
    const int x = P.bx[j * nb + i], y = P.by[j * nb + i];
    uint8_t* f0 = c[0].s + (size_t)(lt - 1) * pf + (size_t)j * nb + i;
    uint8_t* f1 = c[1].s + (size_t)(lt - 1) * pf + (size_t)j * nb + i;
    scee_propose2<MAXRM>(c[0], q[0], q[1], 0, lt, x, y, f0, c[0].tk[i], c[0].tu[i], lb0 + i, ss, pair);
    scee_propose2<MAXRM>(c[1], q[1], q[0], 1, lt, x, y, f1, c[1].tk[i], c[1].tu[i], lb1 + i, ss, pair);
  }
  if (threadIdx.x == 0) {
    c[0].ctl->log_pos += nb;
    c[1].ctl->log_pos += nb;
  }
  finish_tape(c[0], nb);
  finish_tape(c[1], nb);
  __syncthreads();
}

// All bonds of slice lt (t-UV), both replicas alternating per bond, the tape
// slices loaded in chunks of Ns proposals
template <int MAXRM, int KIND, class T, class KT>
__device__ void scee_layer_tuv(Ctx<KIND, T, KT, T, KT>* c, const SceeChain<T>* q, int lt, bool fwd,
                               SceeSmem2<T>& ss, int pair) {
  const SweepParams& P = c[0].P;
  const int N = P.Ns, Nt = P.Nt, pf = P.n_field;
  const uint32_t qs = fwd ? (uint32_t)(lt - 1) * pf : (uint32_t)(Nt + (Nt - lt)) * pf;
  for (int c0 = 0; c0 < pf; c0 += N) {
    const int n = min(N, pf - c0);
    load_tape(c[0], qs + c0, n);
    load_tape(c[1], qs + c0, n);
    const long long lb0 = c[0].ctl->log_pos, lb1 = c[1].ctl->log_pos;
    for (int i = 0; i < n; ++i) {
      const int b = c0 + i, x = P.bx[b], y = P.by[b];
      uint8_t* f0 = c[0].s + (size_t)(lt - 1) * pf + b;
      uint8_t* f1 = c[1].s + (size_t)(lt - 1) * pf + b;
      scee_propose2<MAXRM>(c[0], q[0], q[1], 0, lt, x, y, f0, c[0].tk[i], c[0].tu[i], lb0 + i, ss, pair);
      scee_propose2<MAXRM>(c[1], q[1], q[0], 1, lt, x, y, f1, c[1].tk[i], c[1].tu[i], lb1 + i, ss, pair);
    }
    if (threadIdx.x == 0) {
      c[0].ctl->log_pos += n;
      c[1].ctl->log_pos += n;
    }
    finish_tape(c[0], n);
    finish_tape(c[1], n);
    __syncthreads();
  }
}

template <int KIND, class T>
struct SceeSmemOf { using type = SceeSmem<T>; };
template <class T>
struct SceeSmemOf<KDQ_TV, T> { using type = SceeSmem2<T>; };
template <class T>
struct SceeSmemOf<KDQ_TUV, T> { using type = SceeSmem2<T>; };

template <int MAXRM, int KIND, class T, class KT>
__global__ void __launch_bounds__(KDQ_THREADS, 2) k_scee(const SweepParams P, int mode, int k) {
  extern __shared__ double dyn_d[];
  __shared__ Smem<T> sm;
  const int pair = blockIdx.x;
  const int N = P.Ns;
  // dynamic shared memory: the two replicas' tape slices, then SceeSmem
  using SS = typename SceeSmemOf<KIND, T>::type;
  SS& ss = *reinterpret_cast<SS*>(reinterpret_cast<unsigned char*>(dyn_d) + scee_tape_bytes(N));
  PhaseClock clk;
  clk.start(nullptr);
  const int nrep = P.scee_dop ? 1 : 2;
  auto mk = [&](int r) {
    const int chain = nrep * pair + (r < nrep ? r : 0);
    const size_t cNN = (size_t)chain * P.sz_NN, cNn = (size_t)chain * P.sz_Nn;
    double* tu = dyn_d + (size_t)r * N;
    uint8_t* tk = reinterpret_cast<uint8_t*>(dyn_d + 2 * (size_t)N) + (size_t)r * N;
    return Ctx<KIND, T, KT, T, KT>{P, sm, tk, tu, chain, P.ctl + chain,
                                      static_cast<T*>(P.G) + cNN, static_cast<T*>(P.W1) + cNN,
                                      static_cast<T*>(P.W2) + cNN, static_cast<T*>(P.Yw) + cNn,
                                      static_cast<T*>(P.Y2w) + cNn, static_cast<T*>(P.Y) + cNn,
                                      static_cast<T*>(P.Y2) + cNn, static_cast<T*>(P.Gd) + cNN,
                                      static_cast<T*>(P.Mss) + (size_t)chain * P.sz_nn,
                                      static_cast<T*>(P.X) + cNn, P.piv + (size_t)chain * (N / 2),
                                      P.s + (size_t)chain * P.Nt * P.n_field,
                                      static_cast<const KT*>(P.eK), static_cast<const KT*>(P.eKinv),
                                      static_cast<const KT*>(P.HalfeK), static_cast<const KT*>(P.HalfeKinv),
                                      static_cast<const KT*>(P.K), clk};
  };
  Ctx<KIND, T, KT, T, KT> c[2] = {mk(0), mk(1)};
  const SceeChain<T> q[2] = {scee_chain<T>(P, nrep * pair), scee_chain<T>(P, nrep * pair + nrep - 1)};
  const int NN = P.NN, Th = NN / 2 + 1;
  if (mode == KDQ_MODE_INIT) {
    // block products, both stabilised chains, then the state at node 1
    for (int r = 0; r < nrep; ++r) {
      for (int b = 1; b < NN; ++b)
        scee_block_mats<MAXRM>(c[r], b, q[r].BMs + (size_t)(b - 1) * N * N, q[r].BMi + (size_t)(b - 1) * N * N);
      for (int i = 1; i < NN; ++i) {
        scee_bl<MAXRM>(c[r], q[r], NN - i);
        scee_br<MAXRM>(c[r], q[r], i + 1);
      }
    }
    scee_abgm<MAXRM>(c, q, 1, true, pair);
    return;
  }
  const int lo = (int)P.nodes[k - 1], hi = (int)P.nodes[k];
  if (mode == KDQ_MODE_FWD) {   // idx == k while these slices run
    for (int lt = lo + 1; lt <= hi; ++lt) {
      if constexpr (KIND == KDQ_TV) {   // src/tV/SCEE.jl:87-135
        scee_wrapk<MAXRM>(c[0], q[0], true);
        scee_wrapk<MAXRM>(c[1], q[1], true);
        for (int j = P.z - 1; j >= 0; --j) {
          scee_wrapv<MAXRM>(c[0], q[0], lt, j, true);
          scee_wrapv<MAXRM>(c[1], q[1], lt, j, true);
          scee_layer_tv<MAXRM>(c, q, lt, j, true, ss, pair);
        }
        scee_accumulate(P, pair);
      } else if constexpr (KIND == KDQ_TUV) {   // src/tUV/SCEE.jl:108-140
        scee_wrap<MAXRM>(c[0], q[0], lt, true);
        scee_wrap<MAXRM>(c[1], q[1], lt, true);
        scee_layer_tuv<MAXRM>(c, q, lt, true, ss, pair);
        scee_accumulate(P, pair);
      } else {
        scee_wrap<MAXRM>(c[0], q[0], lt, true);
        if (nrep == 2) scee_wrap<MAXRM>(c[1], q[1], lt, true);
        scee_layer<MAXRM>(c, q, lt, true, ss, pair);
      }
    }
    const int idx = k + 1;   // lt == nodes[idx]
    for (int r = 0; r < nrep; ++r) {
      scee_block_mats<MAXRM>(c[r], idx - 1, q[r].BMs + (size_t)(idx - 2) * N * N,
                             q[r].BMi + (size_t)(idx - 2) * N * N);
      for (int i = idx; i <= max(Th, idx); ++i) scee_br<MAXRM>(c[r], q[r], i);
      for (int i = idx - 1; i >= min(Th, idx); --i) scee_bl<MAXRM>(c[r], q[r], i);
    }
    scee_abgm<MAXRM>(c, q, idx, true, pair);
  } else {                      // idx == k+1 while these slices run
    for (int lt = hi; lt > lo; --lt) {
      if constexpr (KIND == KDQ_TV) {   // src/tV/SCEE.jl:258-282: the wraps come before the node step
        for (int j = 0; j < P.z; ++j) {
          scee_layer_tv<MAXRM>(c, q, lt, j, false, ss, pair);
          scee_wrapv<MAXRM>(c[0], q[0], lt, j, false);
          scee_wrapv<MAXRM>(c[1], q[1], lt, j, false);
        }
        scee_wrapk<MAXRM>(c[0], q[0], false);
        scee_wrapk<MAXRM>(c[1], q[1], false);
        scee_accumulate(P, pair);
      } else if constexpr (KIND == KDQ_TUV) {   // src/tUV/SCEE.jl:228-258: the wraps come before the node step
        scee_layer_tuv<MAXRM>(c, q, lt, false, ss, pair);
        scee_accumulate(P, pair);
        scee_wrap<MAXRM>(c[0], q[0], lt, false);
        scee_wrap<MAXRM>(c[1], q[1], lt, false);
      } else {
        scee_layer<MAXRM>(c, q, lt, false, ss, pair);
      }
      if (lt - 1 == lo) {
        const int idx = k;
        for (int r = 0; r < nrep; ++r) {
          scee_block_mats<MAXRM>(c[r], idx, q[r].BMs + (size_t)(idx - 1) * N * N, q[r].BMi + (size_t)(idx - 1) * N * N);
          for (int i = idx; i >= min(Th, idx); --i) scee_bl<MAXRM>(c[r], q[r], i);
          for (int i = idx + 1; i <= max(Th, idx); ++i) scee_br<MAXRM>(c[r], q[r], i);
        }
        scee_abgm<MAXRM>(c, q, idx, false, pair);
      } else if constexpr (KIND == KDQ_TU) {
        scee_wrap<MAXRM>(c[0], q[0], lt, false);
        if (nrep == 2) scee_wrap<MAXRM>(c[1], q[1], lt, false);
      }
    }
    if (k == 1 && threadIdx.x == 0) {   // end of the sweep: one estimator row
      double* dt = P.scee_det + (size_t)pair * 4;
      if (c[0].ctl->obs_slot < P.scee_O_cap) P.scee_O[(size_t)pair * P.scee_O_cap + c[0].ctl->obs_slot] = dt[2] / dt[3];
      c[0].ctl->obs_slot += 1;
      dt[2] = dt[3] = 0.0;
      c[0].ctl->sweep += 1;
      if (nrep == 2) c[1].ctl->sweep += 1;
    }
  }
}

}  // namespace kdq
