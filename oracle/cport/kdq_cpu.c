/*
 * kdq_cpu.c — CPU restatement of the t-V, t-U and t-UV projector-DQMC
 * sweeps, for timing.
 *
 * TEST INFRASTRUCTURE ONLY: the CPU baseline of bench.py and parity tests
 * against the numpy oracle use it; the product never calls it.
 *
 * It follows the reference operation by operation (t-V: dense
 * bond-rotation GEMMs included; t-U and t-UV: complex eK, complex GEMMs), with the
 * same BLAS/LAPACK routines (?gemm, ?gerqf/?orgrq|?ungrq, ?geqrf/?orgqr|
 * ?ungqr, ?getrf/?getrs) taken at run time from an OpenBLAS shared library
 * (numpy's bundled ILP64 build), as Julia's LinearAlgebra does:
 *   t-V phy_update       src/tV/phy_update.jl:1-188
 *       UpdatePhyLayer!  src/tV/phy_update.jl:190-205
 *       phy_measure      src/tV/phy_update.jl:207-314 (xy_i with 3 arguments)
 *       BM_F!, get_r!, WrapV!  src/tV/GreenMatrix.jl:12-38,76-89,99-119
 *   t-U phy_update       src/tU/phy_update.jl:3-152
 *       UpdatePhyLayer!  src/tU/phy_update.jl:256-267
 *       phy_measure      src/tU/phy_update.jl:154-254
 *       BM_F!, get_r!, WrapKV!  src/tU/GreenMatrix.jl:10-27,49-54,56-86
 *   t-UV phy_update      src/tUV/phy_update.jl:1-186
 *       UpdatePhyLayer!  src/tUV/phy_update.jl:188-203
 *       phy_measure      src/tUV/phy_update.jl:205-354
 *       BM_F!, get_r!, WrapKV!  src/tUV/GreenMatrix.jl:10-36,73-89,92-122
 *   Gupdate!, get_G!     src/public/Gupdate.jl:5-11,139-157
 * The proposal stream is an explicit tape (choice index, uniform) in the
 * reference's consumption order.
 */
#include <complex.h>
#include <dlfcn.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t bint; /* ILP64 BLAS integer */

typedef void (*dgemm_t)(const char*, const char*, const bint*, const bint*, const bint*, const double*,
                        const double*, const bint*, const double*, const bint*, const double*, double*,
                        const bint*);
typedef void (*qrf_t)(const bint*, const bint*, double*, const bint*, double*, double*, const bint*, bint*);
typedef void (*orgq_t)(const bint*, const bint*, const bint*, double*, const bint*, const double*, double*,
                       const bint*, bint*);
typedef void (*getrf_t)(const bint*, const bint*, double*, const bint*, bint*, bint*);
typedef void (*getrs_t)(const char*, const bint*, const bint*, const double*, const bint*, const bint*,
                        double*, const bint*, bint*);

static dgemm_t p_dgemm;
static qrf_t p_dgeqrf, p_dgerqf;
static orgq_t p_dorgqr, p_dorgrq;
static getrf_t p_dgetrf;
static getrs_t p_dgetrs;

typedef double _Complex zc;
typedef void (*zgemm_t)(const char*, const char*, const bint*, const bint*, const bint*, const zc*, const zc*,
                        const bint*, const zc*, const bint*, const zc*, zc*, const bint*);
typedef void (*zqrf_t)(const bint*, const bint*, zc*, const bint*, zc*, zc*, const bint*, bint*);
typedef void (*zungq_t)(const bint*, const bint*, const bint*, zc*, const bint*, const zc*, zc*, const bint*,
                        bint*);
typedef void (*zgetrf_t)(const bint*, const bint*, zc*, const bint*, bint*, bint*);
typedef void (*zgetrs_t)(const char*, const bint*, const bint*, const zc*, const bint*, const bint*, zc*,
                         const bint*, bint*);

static zgemm_t p_zgemm;
static zqrf_t p_zgeqrf, p_zgerqf;
static zungq_t p_zungqr, p_zungrq;
static zgetrf_t p_zgetrf;
static zgetrs_t p_zgetrs;

static void* sym(void* h, const char* base) {
  char name[64];
  const char* forms[] = {"scipy_%s_64_", "%s_64_", "%s_"};
  for (int i = 0; i < 3; ++i) {
    snprintf(name, sizeof name, forms[i], base);
    void* p = dlsym(h, name);
    if (p) return p;
  }
  return NULL;
}

/* Load BLAS/LAPACK from an ILP64 OpenBLAS; returns 0 on success. */
int kdq_cpu_load_blas(const char* path) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) return 1;
  p_dgemm = (dgemm_t)sym(h, "dgemm");
  p_dgeqrf = (qrf_t)sym(h, "dgeqrf");
  p_dgerqf = (qrf_t)sym(h, "dgerqf");
  p_dorgqr = (orgq_t)sym(h, "dorgqr");
  p_dorgrq = (orgq_t)sym(h, "dorgrq");
  p_dgetrf = (getrf_t)sym(h, "dgetrf");
  p_dgetrs = (getrs_t)sym(h, "dgetrs");
  p_zgemm = (zgemm_t)sym(h, "zgemm");
  p_zgeqrf = (zqrf_t)sym(h, "zgeqrf");
  p_zgerqf = (zqrf_t)sym(h, "zgerqf");
  p_zungqr = (zungq_t)sym(h, "zungqr");
  p_zungrq = (zungq_t)sym(h, "zungrq");
  p_zgetrf = (zgetrf_t)sym(h, "zgetrf");
  p_zgetrs = (zgetrs_t)sym(h, "zgetrs");
  return !(p_dgemm && p_dgeqrf && p_dgerqf && p_dorgqr && p_dorgrq && p_dgetrf && p_dgetrs && p_zgemm &&
           p_zgeqrf && p_zgerqf && p_zungqr && p_zungrq && p_zgetrf && p_zgetrs);
}

/* C = A B, column-major, A m x k, B k x n */
static void mm(bint m, bint n, bint k, const double* A, bint lda, const double* B, bint ldb, double* C, bint ldc) {
  const double one = 1.0, zero = 0.0;
  p_dgemm("N", "N", &m, &n, &k, &one, A, &lda, B, &ldb, &zero, C, &ldc);
}

typedef struct {
  int Ns, ns, Nt, z, NN, L1, L2, honeycomb;
  const int64_t* nodes;
  const double *alpha, *gamma, *eta, *eK, *eKinv, *HalfeK, *HalfeKinv, *K, *UV;
  const int32_t* bonds; /* 1-based (x, y), (Ns/2)*z pairs, column-major nnidx order */
  double Ht;
  /* buffers */
  double *G, *tmpNN, *BM, *BLs, *BRs, *tmpNn, *tmpnN, *tmpnn, *tmpN, *tau, *work, *G0, *zN;
  bint* ipiv;
  bint lwork;
  /* tape */
  const uint8_t* tk;
  const double* tu;
  size_t tape_len, tape_pos;
  uint8_t* acc_log;
  size_t log_pos;
} St;

static void setD(St* S, int lt, int j, const uint8_t* s, double sign) {
  const int nb = S->Ns / 2;
  for (int i = 0; i < nb; ++i) {
    const int x = S->bonds[2 * (j * nb + i)] - 1, y = S->bonds[2 * (j * nb + i) + 1] - 1;
    const double v = S->alpha[lt - 1] * S->eta[s[(size_t)(lt - 1) * S->z * nb + j * nb + i] - 1];
    S->tmpN[x] = exp(sign * v);
    S->tmpN[y] = exp(sign * -v);
  }
}

/* WrapV!(tmpNN, G, D, UV_j, "B") on matrix X, src/tV/GreenMatrix.jl:110-118 */
static void wrapV(St* S, double* X, int j) {
  const int N = S->Ns;
  const double* UV = S->UV + (size_t)j * N * N;
  mm(N, N, N, UV, N, X, N, S->tmpNN, N);
  mm(N, N, N, S->tmpNN, N, UV, N, X, N);
  for (int c = 0; c < N; ++c)
    for (int r = 0; r < N; ++r) S->tmpNN[r + (size_t)c * N] = S->tmpN[r] * X[r + (size_t)c * N];
  for (int r = 0; r < N; ++r) S->tmpN[r] = 1.0 / S->tmpN[r];
  for (int c = 0; c < N; ++c)
    for (int r = 0; r < N; ++r) X[r + (size_t)c * N] = S->tmpNN[r + (size_t)c * N] * S->tmpN[c];
  mm(N, N, N, UV, N, X, N, S->tmpNN, N);
  mm(N, N, N, S->tmpNN, N, UV, N, X, N);
}

/* BM_F!, src/tV/GreenMatrix.jl:12-38 */
static void BM_F(St* S, const uint8_t* s, int idx) {
  const int N = S->Ns;
  memset(S->tmpNN, 0, sizeof(double) * N * N);
  for (int i = 0; i < N; ++i) S->tmpNN[i + (size_t)i * N] = 1.0;
  for (int lt = (int)S->nodes[idx - 1] + 1; lt <= (int)S->nodes[idx]; ++lt) {
    mm(N, N, N, S->eK, N, S->tmpNN, N, S->BM, N);
    for (int j = S->z - 1; j >= 0; --j) {
      setD(S, lt, j, s, 1.0);
      const double* UV = S->UV + (size_t)j * N * N;
      mm(N, N, N, UV, N, S->BM, N, S->tmpNN, N);
      for (int c = 0; c < N; ++c)
        for (int r = 0; r < N; ++r) S->BM[r + (size_t)c * N] = S->tmpN[r] * S->tmpNN[r + (size_t)c * N];
      mm(N, N, N, UV, N, S->BM, N, S->tmpNN, N);
      memcpy(S->BM, S->tmpNN, sizeof(double) * N * N);
    }
  }
}

/* get_G!, src/public/Gupdate.jl:139-157 */
static int get_G(St* S, const double* BL, const double* BR) {
  const bint N = S->Ns, n = S->ns;
  bint info;
  mm(n, n, N, BL, n, BR, N, S->tmpnn, n);
  p_dgetrf(&n, &n, S->tmpnn, &n, S->ipiv, &info);
  if (info) return 1;
  memcpy(S->tmpnN, BL, sizeof(double) * n * N);
  p_dgetrs("N", &n, &N, S->tmpnn, &n, S->ipiv, S->tmpnN, &n, &info);
  mm(N, N, n, BR, N, S->tmpnN, n, S->G, N);
  for (bint i = 0; i < N * N; ++i) S->G[i] = -S->G[i];
  for (bint i = 0; i < N; ++i) S->G[i + i * N] += 1.0;
  return 0;
}

static void orth_rows(St* S, double* A) { /* gerqf! + orgrq! on n x N */
  const bint n = S->ns, N = S->Ns;
  bint info;
  p_dgerqf(&n, &N, A, &n, S->tau, S->work, &S->lwork, &info);
  p_dorgrq(&n, &N, &n, A, &n, S->tau, S->work, &S->lwork, &info);
}

static void orth_cols(St* S, double* A) { /* geqrf! + orgqr! on N x n */
  const bint n = S->ns, N = S->Ns;
  bint info;
  p_dgeqrf(&N, &n, A, &N, S->tau, S->work, &S->lwork, &info);
  p_dorgqr(&N, &n, &n, A, &N, S->tau, S->work, &S->lwork, &info);
}

/* UpdatePhyLayer! for direction j of slice lt, src/tV/phy_update.jl:190-205 */
static void update_layer(St* S, uint8_t* s, int lt, int j) {
  const int N = S->Ns, nb = N / 2;
  const double h = sqrt(2.0) / 2.0;
  const double uv[2][2] = {{-h, -h}, {-h, h}};
  uint8_t* sl = s + (size_t)(lt - 1) * S->z * nb + (size_t)j * nb;
  for (int i = 0; i < nb; ++i) {
    const int x = S->bonds[2 * (j * nb + i)] - 1, y = S->bonds[2 * (j * nb + i) + 1] - 1;
    const int k = S->tape_pos < S->tape_len ? S->tk[S->tape_pos] : 0;
    const double u = S->tape_pos < S->tape_len ? S->tu[S->tape_pos] : 2.0;
    S->tape_pos++;
    const int sold = sl[i];
    const int sx = k + (k + 1 >= sold ? 2 : 1);
    const double ds = S->alpha[lt - 1] * (S->eta[sx - 1] - S->eta[sold - 1]);
    const double t2[2] = {exp(ds) - 1.0, exp(-ds) - 1.0};
    double q[2][2], D[2][2], r[2][2], gss[2][2];
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) q[a][b] = uv[a][b] * t2[b];
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) D[a][b] = q[a][0] * uv[0][b] + q[a][1] * uv[1][b];
    const int Sx[2] = {x, y};
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) gss[a][b] = S->G[Sx[a] + (size_t)Sx[b] * N];
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) r[a][b] = D[a][b] - (D[a][0] * gss[0][b] + D[a][1] * gss[1][b]);
    r[0][0] += 1.0;
    r[1][1] += 1.0;
    double p = r[0][0] * r[1][1] - r[0][1] * r[1][0];
    const double det = p;
    const double inv[2][2] = {{r[1][1] / det, -r[0][1] / det}, {-r[1][0] / det, r[0][0] / det}};
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b) r[a][b] = inv[a][0] * D[0][b] + inv[a][1] * D[1][b];
    p *= S->gamma[sx - 1] / S->gamma[sold - 1];
    const int acc = u < p;
    if (S->acc_log) S->acc_log[S->log_pos] = (uint8_t)acc;
    S->log_pos++;
    if (acc) {
      /* Gupdate!: zN = r (E_S - G[S,:]); G -= G[:,S] zN */
      for (int c = 0; c < N; ++c)
        for (int a = 0; a < 2; ++a)
          S->zN[a + 2 * c] = -(r[a][0] * S->G[x + (size_t)c * N] + r[a][1] * S->G[y + (size_t)c * N]);
      for (int a = 0; a < 2; ++a) {
        S->zN[a + 2 * x] += r[a][0];
        S->zN[a + 2 * y] += r[a][1];
      }
      double* gx = S->zN + 2 * N;            /* G[:,x], G[:,y] before the update */
      double* gy = gx + N;
      memcpy(gx, S->G + (size_t)x * N, sizeof(double) * N);
      memcpy(gy, S->G + (size_t)y * N, sizeof(double) * N);
      for (int c = 0; c < N; ++c) {
        const double z0 = S->zN[2 * c], z1 = S->zN[2 * c + 1];
        double* col = S->G + (size_t)c * N;
        for (int rr = 0; rr < N; ++rr) col[rr] -= gx[rr] * z0 + gy[rr] * z1;
      }
      sl[i] = (uint8_t)sx;
    }
  }
}

/* phy_measure, src/tV/phy_update.jl:207-314 */
static void measure(St* S, const uint8_t* s, int lt, double* row) {
  const int N = S->Ns, nb = N / 2;
  double* G0 = S->G0;
  memcpy(G0, S->G, sizeof(double) * N * N);
  if (2 * lt > S->Nt) {
    for (int t = lt; t > S->Nt / 2; --t) {
      for (int j = 0; j < S->z; ++j) {
        setD(S, t, j, s, -1.0);
        wrapV(S, G0, j);
      }
      mm(N, N, N, S->eKinv, N, G0, N, S->tmpNN, N);
      mm(N, N, N, S->tmpNN, N, S->eK, N, G0, N);
    }
  } else {
    for (int t = lt + 1; t <= S->Nt / 2; ++t) {
      mm(N, N, N, G0, N, S->eKinv, N, S->tmpNN, N);
      mm(N, N, N, S->eK, N, S->tmpNN, N, G0, N);
      for (int j = S->z - 1; j >= 0; --j) {
        setD(S, t, j, s, 1.0);
        wrapV(S, G0, j);
      }
    }
  }
  mm(N, N, N, S->HalfeK, N, G0, N, S->tmpNN, N);
  mm(N, N, N, S->tmpNN, N, S->HalfeKinv, N, G0, N);
  double ek = 0.0, ev = 0.0;
  for (size_t e = 0; e < (size_t)N * N; ++e) ek += S->K[e] * G0[e];
  for (int b = 0; b < nb * S->z; ++b) {
    const int x = S->bonds[2 * b] - 1, y = S->bonds[2 * b + 1] - 1;
    ev += (1 - G0[x + (size_t)x * N]) * (1 - G0[y + (size_t)y * N]) - G0[x + (size_t)y * N] * G0[y + (size_t)x * N];
  }
  double R0[4] = {0}, R1[4] = {0};
  if (S->honeycomb) {
    const int L1 = S->L1, L2 = S->L2;
#define g(i, j) G0[(i) + (size_t)(j) * N]
    for (int rx = 1; rx <= L1; ++rx)
      for (int ry = 1; ry <= L2; ++ry) {
        double t[4] = {0, 0, 0, 0};
        for (int ix = 1; ix <= L1; ++ix)
          for (int iy = 1; iy <= L2; ++iy) {
            const int jx = (ix + rx - 1) % L1 + 1, jy = (iy + ry - 1) % L2 + 1;
            const int a1 = 2 * (ix + (iy - 1) * L1) - 2, a2 = 2 * (jx + (jy - 1) * L1) - 2;
            const int b1 = a1 + 1, b2 = a2 + 1;
            if (a1 == a2) {
              t[0] += 1 - g(a1, a1);
              t[1] += 1 - g(b1, b1);
            } else {
              t[0] += (1 - g(a1, a1)) * (1 - g(a2, a2)) - g(a1, a2) * g(a2, a1);
              t[1] += (1 - g(b1, b1)) * (1 - g(b2, b2)) - g(b1, b2) * g(b2, b1);
            }
            t[2] += (1 - g(b1, b1)) * (1 - g(a2, a2)) - g(b1, a2) * g(a2, b1);
            t[3] += (1 - g(a1, a1)) * (1 - g(b2, b2)) - g(a1, b2) * g(b2, a1);
          }
        const double ph = cos(2 * M_PI / L1 * rx + 2 * M_PI / L2 * ry);
        for (int q = 0; q < 4; ++q) {
          R0[q] += t[q];
          R1[q] += ph * t[q];
        }
      }
#undef g
    for (int q = 0; q < 4; ++q) {
      R0[q] *= 4.0 / ((double)N * N);
      R1[q] *= 4.0 / ((double)N * N);
    }
  }
  row[0] += S->Ht * ek;
  row[1] += ev;
  for (int q = 0; q < 4; ++q) {
    row[2 + q] += R0[q];
    row[6 + q] += R1[q];
  }
}

static int is_node(const St* S, int lt) {
  for (int k = 0; k < S->NN; ++k)
    if (S->nodes[k] == lt) return 1;
  return 0;
}

/* The reference's phy_update for one t-V chain.  Returns 0 on success. */
int kdq_cpu_tv_phy_update(int Ns, int Nt, int z, int NN, const int64_t* nodes, const double* alpha,
                          const double* gamma, const double* eta, const double* eK, const double* eKinv,
                          const double* HalfeK, const double* HalfeKinv, const double* K, double Ht,
                          const double* Pt, const int32_t* bonds, const double* UV, int L1, int L2,
                          int honeycomb, uint8_t* s, int sweeps, int record, const uint8_t* tape_k,
                          const double* tape_u, size_t tape_len, double* obs, uint8_t* acc_log) {
  if (!p_dgemm || Ns > 256) return 2;
  St S;
  memset(&S, 0, sizeof S);
  S.Ns = Ns; S.ns = Ns / 2; S.Nt = Nt; S.z = z; S.NN = NN; S.L1 = L1; S.L2 = L2; S.honeycomb = honeycomb;
  S.nodes = nodes; S.alpha = alpha; S.gamma = gamma; S.eta = eta; S.eK = eK; S.eKinv = eKinv;
  S.HalfeK = HalfeK; S.HalfeKinv = HalfeKinv; S.K = K; S.UV = UV; S.bonds = bonds; S.Ht = Ht;
  S.tk = tape_k; S.tu = tape_u; S.tape_len = tape_len; S.acc_log = acc_log;
  const size_t NNe = (size_t)Ns * Ns, Nn = (size_t)Ns * S.ns;
  S.lwork = 64 * (bint)Ns;
  double* mem = (double*)calloc(5 * NNe + 2 * (size_t)NN * Nn + 3 * Nn + (size_t)S.ns * S.ns + Ns + S.ns +
                                    (size_t)S.lwork + 4 * (size_t)Ns,
                                sizeof(double));
  S.ipiv = (bint*)calloc(S.ns, sizeof(bint));
  if (!mem || !S.ipiv) return 3;
  double* p = mem;
  S.G = p; p += NNe; S.tmpNN = p; p += NNe; S.BM = p; p += NNe; S.G0 = p; p += NNe; p += NNe;
  S.BLs = p; p += (size_t)NN * Nn; S.BRs = p; p += (size_t)NN * Nn;
  S.tmpNn = p; p += Nn; S.tmpnN = p; p += Nn; p += Nn;
  S.tmpnn = p; p += (size_t)S.ns * S.ns; S.tmpN = p; p += Ns; S.tau = p; p += S.ns;
  S.work = p; p += S.lwork; S.zN = p;
  const int Θidx = NN / 2 + 1;
  /* BRs[1] = Pt; BLs[NN] = Pt' */
  memcpy(S.BRs, Pt, sizeof(double) * Nn);
  double* BLN = S.BLs + (size_t)(NN - 1) * Nn;
  for (int i = 0; i < Ns; ++i)
    for (int c = 0; c < S.ns; ++c) BLN[c + (size_t)i * S.ns] = Pt[i + (size_t)c * Ns];
  for (int idx = NN - 1; idx >= 1; --idx) {
    BM_F(&S, s, idx);
    mm(S.ns, Ns, Ns, S.BLs + (size_t)idx * Nn, S.ns, S.BM, Ns, S.tmpnN, S.ns);
    orth_rows(&S, S.tmpnN);
    memcpy(S.BLs + (size_t)(idx - 1) * Nn, S.tmpnN, sizeof(double) * Nn);
  }
  int idx = 1, rc = 0;
  if (get_G(&S, S.BLs, S.BRs)) rc = 4;
  for (int w = 0; w < sweeps && !rc; ++w) {
    double row[10] = {0};
    int counter = 0;
    for (int lt = 1; lt <= Nt; ++lt) {
      mm(Ns, Ns, Ns, S.G, Ns, eKinv, Ns, S.tmpNN, Ns);
      mm(Ns, Ns, Ns, eK, Ns, S.tmpNN, Ns, S.G, Ns);
      for (int j = z - 1; j >= 0; --j) {
        setD(&S, lt, j, s, 1.0);
        wrapV(&S, S.G, j);
        update_layer(&S, s, lt, j);
      }
      if (record && abs(idx - Θidx) <= 1) {
        measure(&S, s, lt, row);
        counter++;
      }
      if (is_node(&S, lt)) {
        idx += 1;
        BM_F(&S, s, idx - 1);
        mm(Ns, S.ns, Ns, S.BM, Ns, S.BRs + (size_t)(idx - 2) * Nn, Ns, S.tmpNn, Ns);
        orth_cols(&S, S.tmpNn);
        memcpy(S.BRs + (size_t)(idx - 1) * Nn, S.tmpNn, sizeof(double) * Nn);
        if (get_G(&S, S.BLs + (size_t)(idx - 1) * Nn, S.BRs + (size_t)(idx - 1) * Nn)) rc = 4;
      }
    }
    for (int lt = Nt; lt >= 1; --lt) {
      for (int j = 0; j < z; ++j) {
        update_layer(&S, s, lt, j);
        setD(&S, lt, j, s, -1.0);
        wrapV(&S, S.G, j);
      }
      mm(Ns, Ns, Ns, eKinv, Ns, S.G, Ns, S.tmpNN, Ns);
      mm(Ns, Ns, Ns, S.tmpNN, Ns, eK, Ns, S.G, Ns);
      if (record && abs(idx - Θidx) <= 1) {
        measure(&S, s, lt - 1, row);
        counter++;
      }
      if (is_node(&S, lt - 1)) {
        idx -= 1;
        BM_F(&S, s, idx);
        mm(S.ns, Ns, Ns, S.BLs + (size_t)idx * Nn, S.ns, S.BM, Ns, S.tmpnN, S.ns);
        orth_rows(&S, S.tmpnN);
        memcpy(S.BLs + (size_t)(idx - 1) * Nn, S.tmpnN, sizeof(double) * Nn);
        if (get_G(&S, S.BLs + (size_t)(idx - 1) * Nn, S.BRs + (size_t)(idx - 1) * Nn)) rc = 4;
      }
    }
    if (record && obs)
      for (int q = 0; q < 10; ++q) obs[(size_t)w * 10 + q] = row[q] / counter;
  }
  if (S.tape_pos > tape_len) rc = 5;
  free(mem);
  free(S.ipiv);
  return rc;
}

/* ======================================================================
 * t-U (complex) sweep
 * ====================================================================== */

/* C = A B, complex, column-major */
static void zmm(bint m, bint n, bint k, const zc* A, bint lda, const zc* B, bint ldb, zc* C, bint ldc) {
  const zc one = 1.0, zero = 0.0;
  p_zgemm("N", "N", &m, &n, &k, &one, A, &lda, B, &ldb, &zero, C, &ldc);
}

typedef struct {
  int Ns, ns, Nt, NN, L1, L2, honeycomb;
  const int64_t* nodes;
  const double *alpha, *gamma, *eta;
  const zc *eK, *eKinv, *HalfeK, *HalfeKinv, *K;
  double Ht;
  /* t-UV: bond fields (nb = Ns z bonds, 1-based (x, y) pairs in column-major
   * nnidx order), a = V/g, the couplings, and the real (U < 0) branch */
  int uv, real_type, nb;
  const int32_t* bonds;
  double a, U, V;
  double* vphase;
  zc *G, *tmpNN, *BM, *BLs, *BRs, *tmpNn, *tmpnN, *tmpnn, *tmpN, *tau, *work, *G0, *zN, *gcol;
  bint* ipiv;
  bint lwork;
  const uint8_t* tk;
  const double* tu;
  size_t tape_len, tape_pos;
  uint8_t* acc_log;
  size_t log_pos;
} Su;

/* t-UV slice diagonal: v[x] += eta[s[b, lt]], v[y] += a eta[s[b, lt]] over
 * the bonds b, tmpN = exp(i sign v) (complex) or exp(sign v) (real branch);
 * src/tUV/phy_update.jl:68-78,139-149, src/tUV/GreenMatrix.jl:23-33 */
static void uv_setD(Su* S, int lt, const uint8_t* s, double sign) {
  const uint8_t* sl = s + (size_t)(lt - 1) * S->nb;
  memset(S->vphase, 0, sizeof(double) * S->Ns);
  for (int b = 0; b < S->nb; ++b) {
    const double e = S->eta[sl[b] - 1];
    S->vphase[S->bonds[2 * b] - 1] += e;
    S->vphase[S->bonds[2 * b + 1] - 1] += S->a * e;
  }
  for (int i = 0; i < S->Ns; ++i)
    S->tmpN[i] = S->real_type ? (zc)exp(sign * S->vphase[i]) : cexp(I * (sign * S->vphase[i]));
}

/* tmpN[i] = cis(sign * alpha[lt] * eta[s[i, lt]]) (src/tU/phy_update.jl:61-63,123-125) */
static void u_setD(Su* S, int lt, const uint8_t* s, double sign) {
  if (S->uv) {
    uv_setD(S, lt, s, sign);
    return;
  }
  const uint8_t* sl = s + (size_t)(lt - 1) * S->Ns;
  for (int i = 0; i < S->Ns; ++i) S->tmpN[i] = cexp(I * (sign * S->alpha[lt - 1] * S->eta[sl[i] - 1]));
}

/* X[r, c] <- X[r, c] * D[c] after D <- 1 ./ D, from tmpNN = Diagonal(D) X */
static void u_diag_both(Su* S, zc* X) {
  const int N = S->Ns;
  for (int c = 0; c < N; ++c)
    for (int r = 0; r < N; ++r) S->tmpNN[r + (size_t)c * N] = S->tmpN[r] * X[r + (size_t)c * N];
  for (int r = 0; r < N; ++r) S->tmpN[r] = 1.0 / S->tmpN[r];
  for (int c = 0; c < N; ++c)
    for (int r = 0; r < N; ++r) X[r + (size_t)c * N] = S->tmpNN[r + (size_t)c * N] * S->tmpN[c];
}

/* WrapKV!(.., "Forward", "B"), src/tU/GreenMatrix.jl:64-69 */
static void u_wrap_fwd(Su* S, zc* X) {
  const int N = S->Ns;
  zmm(N, N, N, S->eK, N, X, N, S->tmpNN, N);
  zmm(N, N, N, S->tmpNN, N, S->eKinv, N, X, N);
  u_diag_both(S, X);
}

/* WrapKV!(.., "Backward", "B"), src/tU/GreenMatrix.jl:78-83 */
static void u_wrap_bwd(Su* S, zc* X) {
  const int N = S->Ns;
  u_diag_both(S, X);
  zmm(N, N, N, S->eKinv, N, X, N, S->tmpNN, N);
  zmm(N, N, N, S->tmpNN, N, S->eK, N, X, N);
}

/* BM_F!, src/tU/GreenMatrix.jl:10-27 */
static void u_BM_F(Su* S, const uint8_t* s, int idx) {
  const int N = S->Ns;
  memset(S->BM, 0, sizeof(zc) * N * N);
  for (int i = 0; i < N; ++i) S->BM[i + (size_t)i * N] = 1.0;
  for (int lt = (int)S->nodes[idx - 1] + 1; lt <= (int)S->nodes[idx]; ++lt) {
    u_setD(S, lt, s, 1.0);
    zmm(N, N, N, S->eK, N, S->BM, N, S->tmpNN, N);
    for (int c = 0; c < N; ++c)
      for (int r = 0; r < N; ++r) S->BM[r + (size_t)c * N] = S->tmpN[r] * S->tmpNN[r + (size_t)c * N];
  }
}

/* get_G!, src/public/Gupdate.jl:139-157 */
static int u_get_G(Su* S, const zc* BL, const zc* BR) {
  const bint N = S->Ns, n = S->ns;
  bint info;
  zmm(n, n, N, BL, n, BR, N, S->tmpnn, n);
  p_zgetrf(&n, &n, S->tmpnn, &n, S->ipiv, &info);
  if (info) return 1;
  memcpy(S->tmpnN, BL, sizeof(zc) * n * N);
  p_zgetrs("N", &n, &N, S->tmpnn, &n, S->ipiv, S->tmpnN, &n, &info);
  zmm(N, N, n, BR, N, S->tmpnN, n, S->G, N);
  for (bint i = 0; i < N * N; ++i) S->G[i] = -S->G[i];
  for (bint i = 0; i < N; ++i) S->G[i + i * N] += 1.0;
  return 0;
}

static void u_orth_rows(Su* S, zc* A) { /* gerqf! + orgrq! on n x N */
  const bint n = S->ns, N = S->Ns;
  bint info;
  p_zgerqf(&n, &N, A, &n, S->tau, S->work, &S->lwork, &info);
  p_zungrq(&n, &N, &n, A, &n, S->tau, S->work, &S->lwork, &info);
}

static void u_orth_cols(Su* S, zc* A) { /* geqrf! + orgqr! on N x n */
  const bint n = S->ns, N = S->Ns;
  bint info;
  p_zgeqrf(&N, &n, A, &N, S->tau, S->work, &S->lwork, &info);
  p_zungqr(&N, &n, &n, A, &N, S->tau, S->work, &S->lwork, &info);
}

/* UpdatePhyLayer! of slice lt, src/tU/phy_update.jl:256-267, with get_r!
 * (src/tU/GreenMatrix.jl:49-54) and Gupdate! (src/public/Gupdate.jl:5-11) */
static void u_update_layer(Su* S, uint8_t* s, int lt) {
  const int N = S->Ns;
  uint8_t* sl = s + (size_t)(lt - 1) * N;
  for (int i = 0; i < N; ++i) {
    const int k = S->tape_pos < S->tape_len ? S->tk[S->tape_pos] : 0;
    const double u = S->tape_pos < S->tape_len ? S->tu[S->tape_pos] : 2.0;
    S->tape_pos++;
    const int sold = sl[i];
    const int sx = k + (k + 1 >= sold ? 2 : 1);
    const zc delta = cexp(I * (S->alpha[lt - 1] * (S->eta[sx - 1] - S->eta[sold - 1]))) - 1.0;
    const zc pc = 1.0 + delta * (1.0 - S->G[i + (size_t)i * N]);
    const zc r = delta / pc;
    double p = creal(pc) * creal(pc) + cimag(pc) * cimag(pc);
    p *= S->gamma[sx - 1] / S->gamma[sold - 1];
    const int acc = u < p;
    if (S->acc_log) S->acc_log[S->log_pos] = (uint8_t)acc;
    S->log_pos++;
    if (acc) {
      for (int c = 0; c < N; ++c) S->zN[c] = -(r * S->G[i + (size_t)c * N]);
      S->zN[i] += r;
      memcpy(S->gcol, S->G + (size_t)i * N, sizeof(zc) * N);
      for (int c = 0; c < N; ++c) {
        const zc z0 = S->zN[c];
        zc* col = S->G + (size_t)c * N;
        for (int rr = 0; rr < N; ++rr) col[rr] -= S->gcol[rr] * z0;
      }
      sl[i] = (uint8_t)sx;
    }
  }
}

/* t-UV UpdatePhyLayer! of slice lt, src/tUV/phy_update.jl:188-203: one
 * proposal per bond b = (x, y), get_r! (src/tUV/GreenMatrix.jl:73-89) with
 * Delta = diag(exp(i ds) - 1, exp(i a ds) - 1) (exp without i in the real
 * branch), r = I + Delta (I - G_SS), p = |det r|^2 gamma'/gamma (times
 * exp((eta_old - eta_new)(a + 1)) in the real branch), and the rank-2
 * Gupdate! (src/public/Gupdate.jl:5-11) with r <- inv(r) Delta. */
static void uv_update_layer(Su* S, uint8_t* s, int lt) {
  const int N = S->Ns;
  uint8_t* sl = s + (size_t)(lt - 1) * S->nb;
#define G_(i, j) S->G[(i) + (size_t)(j) * N]
  for (int b = 0; b < S->nb; ++b) {
    const int x = S->bonds[2 * b] - 1, y = S->bonds[2 * b + 1] - 1;
    const int k = S->tape_pos < S->tape_len ? S->tk[S->tape_pos] : 0;
    const double u = S->tape_pos < S->tape_len ? S->tu[S->tape_pos] : 2.0;
    S->tape_pos++;
    const int sold = sl[b];
    const int sx = k + (k + 1 >= sold ? 2 : 1);
    const double ds = S->eta[sx - 1] - S->eta[sold - 1];
    zc d0, d1;
    if (S->real_type) {
      d0 = exp(ds) - 1.0;
      d1 = exp(ds * S->a) - 1.0;
    } else {
      d0 = cexp(I * ds) - 1.0;
      d1 = cexp(I * (ds * S->a)) - 1.0;
    }
    const zc r00 = (d0 + -(d0 * G_(x, x))) + 1.0, r01 = -(d0 * G_(x, y));
    const zc r10 = -(d1 * G_(y, x)), r11 = (d1 + -(d1 * G_(y, y))) + 1.0;
    const zc dt = r00 * r11 - r01 * r10;
    double p = S->real_type ? creal(dt) * creal(dt) : creal(dt) * creal(dt) + cimag(dt) * cimag(dt);
    p *= S->gamma[sx - 1] / S->gamma[sold - 1];
    if (S->real_type) p *= exp((S->eta[sold - 1] - S->eta[sx - 1]) * (S->a + 1.0));
    const int acc = u < p;
    if (S->acc_log) S->acc_log[S->log_pos] = (uint8_t)acc;
    S->log_pos++;
    if (acc) {
      /* R = inv(r) Delta: adjugate / det, columns scaled by Delta */
      const zc R00 = (r11 / dt) * d0, R01 = (-r01 / dt) * d1;
      const zc R10 = (-r10 / dt) * d0, R11 = (r00 / dt) * d1;
      zc* z0 = S->zN;      /* zN = -R G[S, :] + R at columns S, two rows */
      zc* z1 = S->zN + N;
      for (int c = 0; c < N; ++c) {
        z0[c] = -(R00 * G_(x, c) + R01 * G_(y, c));
        z1[c] = -(R10 * G_(x, c) + R11 * G_(y, c));
      }
      z0[x] += R00; z1[x] += R10;
      z0[y] += R01; z1[y] += R11;
      zc* gx = S->gcol;
      zc* gy = S->gcol + N;
      memcpy(gx, S->G + (size_t)x * N, sizeof(zc) * N);
      memcpy(gy, S->G + (size_t)y * N, sizeof(zc) * N);
      for (int c = 0; c < N; ++c) {
        const zc a0 = z0[c], a1 = z1[c];
        zc* col = S->G + (size_t)c * N;
        for (int rr = 0; rr < N; ++rr) col[rr] -= gx[rr] * a0 + gy[rr] * a1;
      }
      sl[b] = (uint8_t)sx;
    }
  }
#undef G_
}

/* CDW0, CDW1, SDW0, SDW1 on the honeycomb lattice, not yet divided by Ns^2.
 * Complex branch (src/tU/phy_update.jl:194-235, src/tUV/phy_update.jl:
 * 306-323): only the first term of every correlator line, the
 * `+adjoint(...)` continuation lines being separate statements whose values
 * are discarded.  Real branch (src/tUV/phy_update.jl:296-305): all terms,
 * times 2 for the two spins. */
static void hc_structure_factors(const Su* S, const zc* G0, int real_branch, zc out[4]) {
  const int N = S->Ns, L1 = S->L1, L2 = S->L2;
  zc cdw0 = 0.0, cdw1 = 0.0, sdw0 = 0.0, sdw1 = 0.0;
#define g(i, j) G0[(i) + (size_t)(j) * N]
  for (int rx = 1; rx <= L1; ++rx)
    for (int ry = 1; ry <= L2; ++ry) {
      zc t1 = 0.0, t2 = 0.0;
      for (int ix = 1; ix <= L1; ++ix)
        for (int iy = 1; iy <= L2; ++iy) {
          const int jx = (ix + rx - 1) % L1 + 1, jy = (iy + ry - 1) % L2 + 1;
          const int a1 = 2 * (ix + (iy - 1) * L1) - 2, a2 = 2 * (jx + (jy - 1) * L1) - 2;
          const int b1 = a1 + 1, b2 = a2 + 1;
          const double dl = a1 == a2 ? 1.0 : 0.0;
          if (real_branch) {
            t1 += 2.0 * ((1.0 - g(a1, a1)) * (1.0 - g(a2, a2)) + (dl - g(a1, a2)) * g(a2, a1));
            t1 += 2.0 * ((1.0 - g(b1, b1)) * (1.0 - g(b2, b2)) + (dl - g(b1, b2)) * g(b2, b1));
            t1 -= 2.0 * ((1.0 - g(b1, b1)) * (1.0 - g(a2, a2)) - g(b1, a2) * g(a2, b1));
            t1 -= 2.0 * ((1.0 - g(a1, a1)) * (1.0 - g(b2, b2)) - g(a1, b2) * g(b2, a1));
            t2 += 2.0 * (1.0 - g(a1, a1)) * (1.0 - g(a2, a2));
            t2 += 2.0 * (1.0 - g(b1, b1)) * (1.0 - g(b2, b2));
            t2 -= 2.0 * (1.0 - g(b1, b1)) * (1.0 - g(a2, a2));
            t2 -= 2.0 * (1.0 - g(a1, a1)) * (1.0 - g(b2, b2));
          } else {
            t1 += (1.0 - g(a1, a1)) * (1.0 - g(a2, a2)) + (dl - g(a1, a2)) * g(a2, a1);
            t1 += (1.0 - g(b1, b1)) * (1.0 - g(b2, b2)) + (dl - g(b1, b2)) * g(b2, b1);
            t1 -= (1.0 - g(b1, b1)) * (1.0 - g(a2, a2)) - g(b1, a2) * g(a2, b1);
            t1 -= (1.0 - g(a1, a1)) * (1.0 - g(b2, b2)) - g(a1, b2) * g(b2, a1);
            t2 += (1.0 - g(a1, a1)) * conj(g(a2, a2));
            t2 += (1.0 - g(b1, b1)) * conj(g(b2, b2));
            t2 -= (1.0 - g(a1, a1)) * conj(g(b2, b2));
            t2 -= (1.0 - g(b1, b1)) * conj(g(a2, a2));
          }
        }
      const double ph = cos(2 * M_PI / L1 * rx + 2 * M_PI / L2 * ry);
      cdw0 += t1 + t2;
      cdw1 += ph * (t1 + t2);
      sdw0 += t1 - t2;
      sdw1 += ph * (t1 - t2);
    }
#undef g
  out[0] = cdw0; out[1] = cdw1; out[2] = sdw0; out[3] = sdw1;
}

/* G0 = HalfeK G(tau = Nt/2) HalfeKinv from the current G at slice lt
 * (src/tU/phy_update.jl:161-182, src/tUV/phy_update.jl:214-251) */
static zc* u_half_green(Su* S, const uint8_t* s, int lt) {
  const int N = S->Ns;
  zc* G0 = S->G0;
  memcpy(G0, S->G, sizeof(zc) * N * N);
  if (2 * lt > S->Nt) {
    for (int t = lt; t > S->Nt / 2; --t) {
      u_setD(S, t, s, -1.0);
      u_wrap_bwd(S, G0);
    }
  } else {
    for (int t = lt + 1; t <= S->Nt / 2; ++t) {
      u_setD(S, t, s, 1.0);
      u_wrap_fwd(S, G0);
    }
  }
  zmm(N, N, N, S->HalfeK, N, G0, N, S->tmpNN, N);
  zmm(N, N, N, S->tmpNN, N, S->HalfeKinv, N, G0, N);
  return G0;
}

/* phy_measure, src/tU/phy_update.jl:154-254: Ek, Eu and (honeycomb) the
 * structure factors as the reference accumulates them. */
static void u_measure(Su* S, const uint8_t* s, int lt, double* row) {
  const int N = S->Ns;
  const zc* G0 = u_half_green(S, s, lt);
  zc ks = 0.0, eu = 0.0, sf[4] = {0.0, 0.0, 0.0, 0.0};
  for (size_t e = 0; e < (size_t)N * N; ++e) ks += S->K[e] * G0[e];
  for (int i = 0; i < N; ++i) eu += (1.0 - G0[i + (size_t)i * N]) * conj(G0[i + (size_t)i * N]);
  if (S->honeycomb) hc_structure_factors(S, G0, 0, sf);
  const double n2 = (double)N * N;
  row[0] += -2.0 * S->Ht * creal(ks);
  row[1] += creal(eu);
  for (int q = 0; q < 4; ++q) row[2 + q] += creal(sf[q]) / n2;
}

/* t-UV phy_measure, src/tUV/phy_update.jl:205-354: Ek = 2 Ht Re sum(K .* G0),
 * Eu (:255-266), Ev over the directed bonds (:268-283) and, on the honeycomb
 * lattices, the structure factors (:285-336).  On the square lattices the
 * four structure-factor columns stay 0: the reference's branch for them
 * (:337-352) tests Lattice == "SQUARE" and writes R0/R1, not the returned
 * CDW/SDW values. */
static void uv_measure(Su* S, const uint8_t* s, int lt, double* row) {
  const int N = S->Ns;
  const zc* G0 = u_half_green(S, s, lt);
  zc ks = 0.0, eu = 0.0, ev = 0.0, sf[4] = {0.0, 0.0, 0.0, 0.0};
  for (size_t e = 0; e < (size_t)N * N; ++e) ks += S->K[e] * G0[e];
  for (int i = 0; i < N; ++i) {
    const zc d = G0[i + (size_t)i * N];
    eu += S->real_type ? (1.0 - d) * (1.0 - d) : (1.0 - d) * conj(d);
  }
  for (int b = 0; b < S->nb; ++b) {
    const int x = S->bonds[2 * b] - 1, y = S->bonds[2 * b + 1] - 1;
    const zc gxx = G0[x + (size_t)x * N], gyy = G0[y + (size_t)y * N];
    const zc gxy = G0[x + (size_t)y * N], gyx = G0[y + (size_t)x * N];
    if (S->real_type) {
      ev += 2.0 * ((1.0 - gxx) * (1.0 - gyy) - gxy * gyx);
      ev += 2.0 * (1.0 - gyy) * (1.0 - gxx);
    } else {
      ev += (1.0 - gxx) * (1.0 - gyy) - gxy * gyx;
      ev += conj(gxx * gyy - gxy * gyx);
      ev += (1.0 - gyy) * conj(gxx) + (1.0 - gxx) * conj(gyy);
    }
  }
  if (S->honeycomb) hc_structure_factors(S, G0, S->real_type, sf);
  const double n2 = (double)N * N;
  row[0] += 2.0 * S->Ht * creal(ks);
  row[1] += S->U * creal(eu);
  row[2] += S->V * creal(ev);
  for (int q = 0; q < 4; ++q) row[3 + q] += creal(sf[q]) / n2;
}

static int u_is_node(const Su* S, int lt) {
  for (int k = 0; k < S->NN; ++k)
    if (S->nodes[k] == lt) return 1;
  return 0;
}

/* Measurement window at stabilisation index idx: t-U measures at
 * Thidx - idx in {0, 1} going forward and idx - Thidx in {0, 1} going back
 * (src/tU/phy_update.jl:69,112); t-UV at |idx - Thidx| <= 1 both ways
 * (src/tUV/phy_update.jl:83,127). */
static int u_window(const Su* S, int idx, int forward) {
  const int th = S->NN / 2 + 1;
  if (S->uv) return idx - th >= -1 && idx - th <= 1;
  const int d = forward ? th - idx : idx - th;
  return d >= 0 && d <= 1;
}

/* The sweep driver shared by t-U and t-UV: chain set-up (BLs from Pt'),
 * Sweeps forward+backward passes with wraps, local updates, measurements and
 * QR-stabilised recomputes at the nodes (src/tU/phy_update.jl:3-152,
 * src/tUV/phy_update.jl:1-186).  Pt: Ns x ns complex, column-major.
 * obs: nobs doubles per sweep. */
static int u_drive(Su* S, const zc* P, uint8_t* s, int sweeps, int record, double* obs, int nobs) {
  const int Ns = S->Ns, NN = S->NN, Nt = S->Nt;
  const size_t NNe = (size_t)Ns * Ns, Nn = (size_t)Ns * S->ns;
  S->lwork = 64 * (bint)Ns;
  zc* mem = (zc*)calloc(4 * NNe + 2 * (size_t)NN * Nn + 2 * Nn + (size_t)S->ns * S->ns + Ns + S->ns +
                            (size_t)S->lwork + 4 * (size_t)Ns,
                        sizeof(zc));
  S->vphase = (double*)calloc(Ns, sizeof(double));
  S->ipiv = (bint*)calloc(S->ns, sizeof(bint));
  if (!mem || !S->ipiv || !S->vphase) {
    free(mem);
    free(S->ipiv);
    free(S->vphase);
    return 3;
  }
  zc* p = mem;
  S->G = p; p += NNe; S->tmpNN = p; p += NNe; S->BM = p; p += NNe; S->G0 = p; p += NNe;
  S->BLs = p; p += (size_t)NN * Nn; S->BRs = p; p += (size_t)NN * Nn;
  S->tmpNn = p; p += Nn; S->tmpnN = p; p += Nn;
  S->tmpnn = p; p += (size_t)S->ns * S->ns; S->tmpN = p; p += Ns; S->tau = p; p += S->ns;
  S->work = p; p += S->lwork; S->zN = p; p += 2 * (size_t)Ns; S->gcol = p;
  /* BRs[1] = Pt; BLs[NN] = Pt' (adjoint) */
  memcpy(S->BRs, P, sizeof(zc) * Nn);
  zc* BLN = S->BLs + (size_t)(NN - 1) * Nn;
  for (int i = 0; i < Ns; ++i)
    for (int c = 0; c < S->ns; ++c) BLN[c + (size_t)i * S->ns] = conj(P[i + (size_t)c * Ns]);
  for (int idx = NN - 1; idx >= 1; --idx) {
    u_BM_F(S, s, idx);
    zmm(S->ns, Ns, Ns, S->BLs + (size_t)idx * Nn, S->ns, S->BM, Ns, S->tmpnN, S->ns);
    u_orth_rows(S, S->tmpnN);
    memcpy(S->BLs + (size_t)(idx - 1) * Nn, S->tmpnN, sizeof(zc) * Nn);
  }
  int idx = 1, rc = 0;
  if (u_get_G(S, S->BLs, S->BRs)) rc = 4;
  for (int w = 0; w < sweeps && !rc; ++w) {
    double row[7] = {0};
    int counter = 0;
    for (int lt = 1; lt <= Nt; ++lt) {
      u_setD(S, lt, s, 1.0);
      u_wrap_fwd(S, S->G);
      if (S->uv)
        uv_update_layer(S, s, lt);
      else
        u_update_layer(S, s, lt);
      if (record && u_window(S, idx, 1)) {
        if (S->uv)
          uv_measure(S, s, lt, row);
        else
          u_measure(S, s, lt, row);
        counter++;
      }
      if (u_is_node(S, lt)) {
        idx += 1;
        u_BM_F(S, s, idx - 1);
        zmm(Ns, S->ns, Ns, S->BM, Ns, S->BRs + (size_t)(idx - 2) * Nn, Ns, S->tmpNn, Ns);
        u_orth_cols(S, S->tmpNn);
        memcpy(S->BRs + (size_t)(idx - 1) * Nn, S->tmpNn, sizeof(zc) * Nn);
        if (u_get_G(S, S->BLs + (size_t)(idx - 1) * Nn, S->BRs + (size_t)(idx - 1) * Nn)) rc = 4;
      }
    }
    for (int lt = Nt; lt >= 1; --lt) {
      if (S->uv)
        uv_update_layer(S, s, lt);
      else
        u_update_layer(S, s, lt);
      if (record && u_window(S, idx, 0)) {
        if (S->uv)
          uv_measure(S, s, lt, row);
        else
          u_measure(S, s, lt, row);
        counter++;
      }
      u_setD(S, lt, s, -1.0);
      u_wrap_bwd(S, S->G);
      if (u_is_node(S, lt - 1)) {
        idx -= 1;
        u_BM_F(S, s, idx);
        zmm(S->ns, Ns, Ns, S->BLs + (size_t)idx * Nn, S->ns, S->BM, Ns, S->tmpnN, S->ns);
        u_orth_rows(S, S->tmpnN);
        memcpy(S->BLs + (size_t)(idx - 1) * Nn, S->tmpnN, sizeof(zc) * Nn);
        if (u_get_G(S, S->BLs + (size_t)(idx - 1) * Nn, S->BRs + (size_t)(idx - 1) * Nn)) rc = 4;
      }
    }
    if (record && obs)
      for (int q = 0; q < nobs; ++q) obs[(size_t)w * nobs + q] = counter ? row[q] / counter : 0.0;
  }
  if (S->tape_pos > S->tape_len) rc = 5;
  free(mem);
  free(S->ipiv);
  free(S->vphase);
  return rc;
}

/* The reference's phy_update for one t-U chain (complex matrices as
 * interleaved (re, im) doubles).  obs: 6 doubles per sweep.  Returns 0 on
 * success. */
int kdq_cpu_tu_phy_update(int Ns, int Nt, int NN, const int64_t* nodes, const double* alpha, const double* gamma,
                          const double* eta, const double* eK, const double* eKinv, const double* HalfeK,
                          const double* HalfeKinv, const double* K, double Ht, const double* Pt, int L1, int L2,
                          int honeycomb, uint8_t* s, int sweeps, int record, const uint8_t* tape_k,
                          const double* tape_u, size_t tape_len, double* obs, uint8_t* acc_log) {
  if (!p_zgemm || Ns > 512) return 2;
  Su S;
  memset(&S, 0, sizeof S);
  S.Ns = Ns; S.ns = Ns / 2; S.Nt = Nt; S.NN = NN; S.L1 = L1; S.L2 = L2; S.honeycomb = honeycomb;
  S.nodes = nodes; S.alpha = alpha; S.gamma = gamma; S.eta = eta;
  S.eK = (const zc*)eK; S.eKinv = (const zc*)eKinv; S.HalfeK = (const zc*)HalfeK;
  S.HalfeKinv = (const zc*)HalfeKinv; S.K = (const zc*)K; S.Ht = Ht;
  S.tk = tape_k; S.tu = tape_u; S.tape_len = tape_len; S.acc_log = acc_log;
  return u_drive(&S, (const zc*)Pt, s, sweeps, record, obs, 6);
}

/* The reference's phy_update for one t-UV chain (src/tUV/phy_update.jl:
 * 1-186).  Matrices are complex (interleaved (re, im) doubles) in both
 * branches; real_type = 1 (U < 0, the reference's Float64 sweep) takes real
 * exponentials, det^2 weights with the exp((eta_old - eta_new)(a + 1))
 * factor and the real measurement formulas, whose values the complex
 * storage carries with zero imaginary parts.  bonds: nb = Ns z 1-based
 * (x, y) pairs in column-major nnidx order; s: nb x Nt.  obs: 7 doubles per
 * sweep.  Returns 0 on success. */
int kdq_cpu_tuv_phy_update(int Ns, int Nt, int NN, const int64_t* nodes, const double* gamma, const double* eta,
                           const double* eK, const double* eKinv, const double* HalfeK, const double* HalfeKinv,
                           const double* K, double Ht, double U, double V, double a, int real_type,
                           const double* Pt, const int32_t* bonds, int nb, int L1, int L2, int honeycomb,
                           uint8_t* s, int sweeps, int record, const uint8_t* tape_k, const double* tape_u,
                           size_t tape_len, double* obs, uint8_t* acc_log) {
  if (!p_zgemm || Ns > 512) return 2;
  Su S;
  memset(&S, 0, sizeof S);
  S.Ns = Ns; S.ns = Ns / 2; S.Nt = Nt; S.NN = NN; S.L1 = L1; S.L2 = L2; S.honeycomb = honeycomb;
  S.nodes = nodes; S.gamma = gamma; S.eta = eta;
  S.eK = (const zc*)eK; S.eKinv = (const zc*)eKinv; S.HalfeK = (const zc*)HalfeK;
  S.HalfeKinv = (const zc*)HalfeKinv; S.K = (const zc*)K; S.Ht = Ht;
  S.uv = 1; S.real_type = real_type; S.nb = nb; S.bonds = bonds; S.a = a; S.U = U; S.V = V;
  S.tk = tape_k; S.tu = tape_u; S.tape_len = tape_len; S.acc_log = acc_log;
  return u_drive(&S, (const zc*)Pt, s, sweeps, record, obs, 7);
}
