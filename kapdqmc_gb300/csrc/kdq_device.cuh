// Device building blocks of the sweep: complex arithmetic, block-level
// FP64 GEMM, Householder orthonormalisation, LU solve and reductions.
//
// Every routine here is executed by a whole CTA (all threads call it, with
// identical arguments) and works on column-major matrices addressed through
// generic pointers, so the same code runs on shared or global memory.  A
// routine ends with __syncthreads() so its result is visible to the caller.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

// Largest order whose Gauss-Jordan / Cholesky determinant bookkeeping is
// deferred past the pivot loop (the sweep's ns <= 96, SCEE regions <= 96).
constexpr int GJ_DEFER_MAX = 96;

namespace kdq {

// ---------------------------------------------------------------- complex
struct cd {
  double x, y;
};

__host__ __device__ inline cd mkc(double x, double y) { return cd{x, y}; }
__device__ inline cd operator+(cd a, cd b) { return {a.x + b.x, a.y + b.y}; }
__device__ inline cd operator-(cd a, cd b) { return {a.x - b.x, a.y - b.y}; }
__device__ inline cd operator-(cd a) { return {-a.x, -a.y}; }
__device__ inline cd operator*(cd a, cd b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ inline cd operator*(cd a, double b) { return {a.x * b, a.y * b}; }
__device__ inline cd operator*(double a, cd b) { return {a * b.x, a * b.y}; }
__device__ inline cd operator/(cd a, cd b) {
  // Smith's algorithm (scaled division), avoids overflow of |b|^2.
  if (fabs(b.x) >= fabs(b.y)) {
    double r = b.y / b.x, d = b.x + r * b.y;
    return {(a.x + a.y * r) / d, (a.y - a.x * r) / d};
  }
  double r = b.x / b.y, d = b.y + r * b.x;
  return {(a.x * r + a.y) / d, (a.y * r - a.x) / d};
}
__device__ inline cd operator/(cd a, double b) { return {a.x / b, a.y / b}; }
__device__ inline cd conjg(cd a) { return {a.x, -a.y}; }
__device__ inline double conjg(double a) { return a; }
__device__ inline double re(cd a) { return a.x; }
__device__ inline double re(double a) { return a; }
__device__ inline double abs2(cd a) { return a.x * a.x + a.y * a.y; }
__device__ inline double abs2(double a) { return a * a; }
__device__ inline bool finite(cd a) { return isfinite(a.x) && isfinite(a.y); }
__device__ inline bool finite(double a) { return isfinite(a); }

// complex float (working precision of the mixed-precision sweep)
struct cf {
  float x, y;
};
__device__ inline cf operator+(cf a, cf b) { return {a.x + b.x, a.y + b.y}; }
__device__ inline cf operator-(cf a, cf b) { return {a.x - b.x, a.y - b.y}; }
__device__ inline cf operator-(cf a) { return {-a.x, -a.y}; }
__device__ inline cf operator*(cf a, cf b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
__device__ inline cf operator*(cf a, float b) { return {a.x * b, a.y * b}; }
__device__ inline cf operator*(float a, cf b) { return {a * b.x, a * b.y}; }
__device__ inline cf operator*(cf a, double b) { return {a.x * (float)b, a.y * (float)b}; }
__device__ inline cf conjg(cf a) { return {a.x, -a.y}; }
__device__ inline float conjg(float a) { return a; }
__device__ inline float re(cf a) { return a.x; }
__device__ inline float re(float a) { return a; }
__device__ inline double abs2(cf a) { return (double)a.x * a.x + (double)a.y * a.y; }
__device__ inline double abs2(float a) { return (double)a * a; }

// ----------------------------------------------------------- double-float
// hi + lo, two floats with |lo| <= ulp(hi)/2: a 48-bit significand carried
// on the FP32 pipe (Dekker, "A floating-point technique for extending the
// available precision", Numer. Math. 18, 1971; error-free sums after Knuth,
// TAOCP vol. 2, 4.2.2; error-free products with a fused multiply-add).  The
// stabilisation type of the mixed-precision sweep: on GB300 the FP32 pipe
// is ~67x the FP64 pipe, so ~15 FP32 operations per multiply-add still run
// several times faster than one DFMA.  The intrinsics keep every rounding
// step explicit (no contraction into FMAs).
struct df {
  float hi, lo;
};
__device__ __forceinline__ df df_fast2(float s, float e) {   // |s| >= |e|
  const float h = __fadd_rn(s, e);
  return {h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ df df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df df_from(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }   // exact
__device__ __forceinline__ df operator+(df a, df b) {
  const df s = df_two_sum(a.hi, b.hi);
  return df_fast2(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df operator-(df a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df_fast2(p, e);
}
__device__ __forceinline__ df operator*(df a, double b) { return a * df_from(b); }
__device__ __forceinline__ df operator*(double a, df b) { return df_from(a) * b; }
__device__ __forceinline__ df operator/(df a, double b) { return df_from(df_to(a) / b); }
__device__ __forceinline__ df operator/(df a, df b) { return df_from(df_to(a) / df_to(b)); }
// acc += a * b in one renormalisation (15 FP32 operations)
__device__ __forceinline__ void madd(df& acc, df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const df s = df_two_sum(acc.hi, p);
  acc = df_fast2(s.hi, __fadd_rn(s.lo, __fadd_rn(e, acc.lo)));
}
// acc += a * b without the final renormalisation (12 FP32 operations):
// acc.hi is the rounded running sum, acc.lo collects the rounding errors;
// normalise(acc) before acc is used as an operand.
__device__ __forceinline__ void madd_lazy(df& acc, df a, df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  const df s = df_two_sum(acc.hi, p);
  acc.hi = s.hi;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(s.lo, e));
}
__device__ __forceinline__ df normalise(df a) { return df_two_sum(a.hi, a.lo); }
__device__ __forceinline__ df conjg(df a) { return a; }
__device__ __forceinline__ double re(df a) { return df_to(a); }
__device__ __forceinline__ double abs2(df a) { const double v = df_to(a); return v * v; }

// complex double-float
struct cdf {
  df x, y;
};
__device__ __forceinline__ cdf operator+(cdf a, cdf b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cdf operator-(cdf a, cdf b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cdf operator-(cdf a) { return {-a.x, -a.y}; }
__device__ __forceinline__ cdf operator*(cdf a, cdf b) {
  df re_ = a.x * b.x, im_ = a.x * b.y;
  madd(re_, -a.y, b.y);
  madd(im_, a.y, b.x);
  return {re_, im_};
}
__device__ __forceinline__ cdf operator*(cdf a, double b) { const df d = df_from(b); return {a.x * d, a.y * d}; }
__device__ __forceinline__ cdf operator*(double a, cdf b) { return b * a; }
__device__ __forceinline__ cdf operator/(cdf a, double b) { return {a.x / b, a.y / b}; }
__device__ __forceinline__ cdf conjg(cdf a) { return {a.x, -a.y}; }
// quotients are rare (pivots, reflector scalars): through complex128
__device__ inline cdf cdf_from(cd v) { return {df_from(v.x), df_from(v.y)}; }
__device__ inline cdf operator/(cdf a, cdf b) {
  return cdf_from(cd{df_to(a.x), df_to(a.y)} / cd{df_to(b.x), df_to(b.y)});
}
__device__ __forceinline__ double re(cdf a) { return df_to(a.x); }
__device__ __forceinline__ double abs2(cdf a) {
  const double u = df_to(a.x), v = df_to(a.y);
  return u * u + v * v;
}
// complex multiply-add, lazily accumulated (see madd_lazy): normalise the
// accumulator before it is used as an operand
__device__ __forceinline__ void madd(cdf& acc, cdf a, cdf b) {
  madd_lazy(acc.x, a.x, b.x);
  madd_lazy(acc.x, -a.y, b.y);
  madd_lazy(acc.y, a.x, b.y);
  madd_lazy(acc.y, a.y, b.x);
}
__device__ __forceinline__ cdf normalise(cdf a) { return {normalise(a.x), normalise(a.y)}; }
__device__ __forceinline__ void madd(cdf& acc, cdf a, df b) {
  madd(acc.x, a.x, b);
  madd(acc.y, a.y, b);
}
__device__ __forceinline__ void madd(cdf& acc, df a, cdf b) {
  madd(acc.x, a, b.x);
  madd(acc.y, a, b.y);
}

// conversions between the FP64 and the working types
template <class To> struct cvt_t;
template <> struct cvt_t<double> {
  __device__ static double f(double v) { return v; }
  __device__ static double f(float v) { return v; }
  __device__ static double f(df v) { return df_to(v); }
};
template <> struct cvt_t<float> {
  __device__ static float f(double v) { return (float)v; }
  __device__ static float f(float v) { return v; }
  __device__ static float f(df v) { return __fadd_rn(v.hi, v.lo); }
};
template <> struct cvt_t<cd> {
  __device__ static cd f(cd v) { return v; }
  __device__ static cd f(cf v) { return {v.x, v.y}; }
  __device__ static cd f(double v) { return {v, 0.0}; }
  __device__ static cd f(float v) { return {v, 0.0}; }
  __device__ static cd f(cdf v) { return {df_to(v.x), df_to(v.y)}; }
  __device__ static cd f(df v) { return {df_to(v), 0.0}; }
};
template <> struct cvt_t<cf> {
  __device__ static cf f(cf v) { return v; }
  __device__ static cf f(cd v) { return {(float)v.x, (float)v.y}; }
  __device__ static cf f(double v) { return {(float)v, 0.0f}; }
  __device__ static cf f(float v) { return {v, 0.0f}; }
  __device__ static cf f(cdf v) { return {__fadd_rn(v.x.hi, v.x.lo), __fadd_rn(v.y.hi, v.y.lo)}; }
};
template <> struct cvt_t<df> {
  __device__ static df f(df v) { return v; }
  __device__ static df f(double v) { return df_from(v); }
  __device__ static df f(float v) { return {v, 0.0f}; }
};
template <> struct cvt_t<cdf> {
  __device__ static cdf f(cdf v) { return v; }
  __device__ static cdf f(cd v) { return {df_from(v.x), df_from(v.y)}; }
  __device__ static cdf f(cf v) { return {{v.x, 0.0f}, {v.y, 0.0f}}; }
  __device__ static cdf f(double v) { return {df_from(v), {0.0f, 0.0f}}; }
  __device__ static cdf f(float v) { return {{v, 0.0f}, {0.0f, 0.0f}}; }
};
template <class To, class From> __device__ inline To cvt(From v) { return cvt_t<To>::f(v); }

// the reduced-precision type of an FP64 type
template <class T> struct low_t;
template <> struct low_t<double> { using type = float; };
template <> struct low_t<cd> { using type = cf; };

// the double-float type standing in for an FP64 type
template <class T> struct dfl_t;
template <> struct dfl_t<double> { using type = df; };
template <> struct dfl_t<cd> { using type = cdf; };

template <class T> __device__ inline T zero();
template <> __device__ inline df zero<df>() { return {0.0f, 0.0f}; }
template <> __device__ inline cdf zero<cdf>() { return {{0.0f, 0.0f}, {0.0f, 0.0f}}; }
template <> __device__ inline double zero<double>() { return 0.0; }
template <> __device__ inline cd zero<cd>() { return {0.0, 0.0}; }
template <> __device__ inline float zero<float>() { return 0.0f; }
template <> __device__ inline cf zero<cf>() { return {0.0f, 0.0f}; }
template <class T> __device__ inline T one();
template <> __device__ inline df one<df>() { return {1.0f, 0.0f}; }
template <> __device__ inline cdf one<cdf>() { return {{1.0f, 0.0f}, {0.0f, 0.0f}}; }
template <> __device__ inline double one<double>() { return 1.0; }
template <> __device__ inline cd one<cd>() { return {1.0, 0.0}; }
template <> __device__ inline float one<float>() { return 1.0f; }
template <> __device__ inline cf one<cf>() { return {1.0f, 0.0f}; }
template <class T> __device__ inline T from_real(double v);
template <> __device__ inline df from_real<df>(double v) { return df_from(v); }
template <> __device__ inline cdf from_real<cdf>(double v) { return {df_from(v), {0.0f, 0.0f}}; }
template <> __device__ inline double from_real<double>(double v) { return v; }
template <> __device__ inline cd from_real<cd>(double v) { return {v, 0.0}; }
template <> __device__ inline float from_real<float>(double v) { return (float)v; }
template <> __device__ inline cf from_real<cf>(double v) { return {(float)v, 0.0f}; }

// acc += a * b for every mix of real and complex operands
__device__ inline void madd(double& acc, double a, double b) { acc = fma(a, b, acc); }
__device__ inline void madd(cd& acc, cd a, double b) { acc.x = fma(a.x, b, acc.x); acc.y = fma(a.y, b, acc.y); }
__device__ inline void madd(cd& acc, double a, cd b) { acc.x = fma(a, b.x, acc.x); acc.y = fma(a, b.y, acc.y); }
__device__ inline void madd(cd& acc, cd a, cd b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}

__device__ inline void madd(float& acc, float a, float b) { acc = fmaf(a, b, acc); }
__device__ inline void madd(cf& acc, cf a, float b) { acc.x = fmaf(a.x, b, acc.x); acc.y = fmaf(a.y, b, acc.y); }
__device__ inline void madd(cf& acc, float a, cf b) { acc.x = fmaf(a, b.x, acc.x); acc.y = fmaf(a, b.y, acc.y); }
__device__ inline void madd(cf& acc, cf a, cf b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}

template <class T> struct conv;
template <> struct conv<double> {
  __device__ static double from(double v) { return v; }
};
template <> struct conv<cd> {
  __device__ static cd from(double v) { return {v, 0.0}; }
  __device__ static cd from(cd v) { return v; }
};

// ------------------------------------------------------------- reductions
__device__ inline double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ inline cd warp_sum(cd v) { return {warp_sum(v.x), warp_sum(v.y)}; }
__device__ inline float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ inline cf warp_sum(cf v) { return {warp_sum(v.x), warp_sum(v.y)}; }
__device__ inline df warp_sum(df v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const df w = {__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
    v = v + w;
  }
  return v;
}
__device__ inline cdf warp_sum(cdf v) { return {warp_sum(v.x), warp_sum(v.y)}; }

// Block-wide sum; `red` is shared scratch of >= 32 doubles.  All threads
// receive the result.
__device__ inline double block_sum(double v, double* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < nw; ++w) t += red[w];
  __syncthreads();
  return t;
}

// accumulators of the FP64, FP32 and complex types need no normalisation
__device__ __forceinline__ double normalise(double a) { return a; }
__device__ __forceinline__ float normalise(float a) { return a; }
__device__ __forceinline__ cd normalise(cd a) { return a; }
__device__ __forceinline__ cf normalise(cf a) { return a; }

// ------------------------------------------------------------------- GEMM
// C[M x N] = A[M x K] * B[K x N] (column-major, C must not alias A or B),
// with an optional epilogue C[i,j] = rs[i] * acc * cs[j]; with SUB the
// result is subtracted from C instead (C -= A B).
// Register-tiled: the M x N output is cut into RS x CS micro-
// tiles of TM x TN (RS = ceil(M/TM), CS = ceil(N/TN)); thread t owns the
// micro-tile (t mod RS, t div RS) with rows r + RS*m and columns c + CS*n,
// so consecutive lanes load consecutive rows of A and the B values of a
// warp are near-broadcasts.  When RS*CS is a multiple of 32 no FP64 lane is
// wasted (the FP64 pipe, not memory, bounds these products on GB300).
template <int TM, int TN, class TA, class TB, class TC, class TS = double, bool SUB = false>
__device__ void bgemm_t(int M, int N, int K, const TA* __restrict__ A, int lda,
                        const TB* __restrict__ B, int ldb, TC* __restrict__ C, int ldc,
                        const TS* rs = nullptr, const TS* cs = nullptr) {
  const int RS = (M + TM - 1) / TM, CS = (N + TN - 1) / TN;
  const int tiles = RS * CS;
  for (int t = threadIdx.x; t < tiles; t += blockDim.x) {
    const int r0 = t % RS, c0 = t / RS;
    TC acc[TM][TN];
#pragma unroll
    for (int m = 0; m < TM; ++m)
#pragma unroll
      for (int n = 0; n < TN; ++n) acc[m][n] = zero<TC>();
    int rows[TM], cols[TN];
#pragma unroll
    for (int m = 0; m < TM; ++m) rows[m] = min(r0 + RS * m, M - 1);
#pragma unroll
    for (int n = 0; n < TN; ++n) cols[n] = min(c0 + CS * n, N - 1);
    for (int k = 0; k < K; ++k) {
      TA a[TM];
      TB b[TN];
#pragma unroll
      for (int m = 0; m < TM; ++m) a[m] = A[rows[m] + (size_t)k * lda];
#pragma unroll
      for (int n = 0; n < TN; ++n) b[n] = B[k + (size_t)cols[n] * ldb];
#pragma unroll
      for (int m = 0; m < TM; ++m)
#pragma unroll
        for (int n = 0; n < TN; ++n) madd(acc[m][n], a[m], b[n]);
    }
#pragma unroll
    for (int m = 0; m < TM; ++m) {
      const int i = r0 + RS * m;
      if (i >= M) continue;
#pragma unroll
      for (int n = 0; n < TN; ++n) {
        const int j = c0 + CS * n;
        if (j >= N) continue;
        TC v = normalise(acc[m][n]);
        if (rs) v = rs[i] * v;
        if (cs) v = v * cs[j];
        if constexpr (SUB) v = C[i + (size_t)j * ldc] - v;   // C -= A B
        C[i + (size_t)j * ldc] = v;
      }
    }
  }
  __syncthreads();
}

// ------------------------------------------------ Householder QR (thin Q)
// Columns c0 <= c < n of A (ld N): A[j:,c] -= s w (w^H A[j:,c]) with the
// reflector w = x[j:] and s = 2 / (w^H w).  Warp `warp` of nw takes columns
// c0 + warp, c0 + warp + nw, ... three at a time: the three dot products and
// their warp reductions are independent chains, so they overlap; each
// column's own arithmetic is the same as one column at a time.
template <class T>
__device__ __forceinline__ void reflect_columns(int N, int c0, int n, int j, const T* x, double s, T* A, int warp,
                                                int nw, int lane) {
  for (int c = c0 + warp; c < n; c += 3 * nw) {
    const int cb = c + nw, cc = c + 2 * nw;
    T* ya = A + (size_t)c * N;
    T* yb = A + (size_t)min(cb, n - 1) * N;
    T* yc = A + (size_t)min(cc, n - 1) * N;
    T ta = zero<T>(), tb = zero<T>(), tc = zero<T>();
    for (int i = j + lane; i < N; i += 32) {
      const T xi = conjg(x[i]);
      madd(ta, xi, ya[i]);
      if (cb < n) madd(tb, xi, yb[i]);
      if (cc < n) madd(tc, xi, yc[i]);
    }
    ta = warp_sum(normalise(ta));
    tb = warp_sum(normalise(tb));
    tc = warp_sum(normalise(tc));
    ta = ta * s;
    tb = tb * s;
    tc = tc * s;
    for (int i = j + lane; i < N; i += 32) {
      const T xi = x[i];
      ya[i] = ya[i] - xi * ta;
      if (cb < n) yb[i] = yb[i] - xi * tb;
      if (cc < n) yc[i] = yc[i] - xi * tc;
    }
  }
}

// Overwrites Q (N x n, column-major, ld N) with an orthonormal basis of the
// column space of Y (N x n, ld N), destroying Y.  Reflectors
// H = I - w w^H * (2 / w^H w) with w = x + e^{i arg x0} |x| e1 (Householder
// 1958; the LAPACK ?geqrf + ?orgqr pair restated with Hermitian reflectors).
// Scratch: wn (n doubles: 2/(w^H w)), red (>= 32 doubles) in shared memory.
// The discarded triangle has R_jj = -e^{i arg x0} |x|; when given, log_out and
// phase_out receive sum_j log|R_jj| and prod_j R_jj/|R_jj| (the log-weight
// of the stabilised B chain).
template <class T>
__device__ void householder_q(int N, int n, T* Y, T* Q, double* wn, double* red,
                              double* log_out = nullptr, cd* phase_out = nullptr) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, warp = tid >> 5, nw = nt >> 5;
  double lgs = 0.0;          // sum of log |R_jj| (thread 0)
  cd phs = mkc(1.0, 0.0);    // product of R_jj / |R_jj| (thread 0)
  for (int j = 0; j < n; ++j) {
    T* x = Y + (size_t)j * N;
    double s = 0.0;
    for (int i = j + tid; i < N; i += nt) s += abs2(x[i]);
    const double nrm2 = block_sum(s, red);
    const double nrm = sqrt(nrm2);
    if (tid == 0) {
      T a = x[j];
      double aa = sqrt(abs2(a));
      T ph = aa > 0.0 ? a / aa : one<T>();
      T wj = a + ph * nrm;                    // w_j
      double ww = 2.0 * nrm * (nrm + aa);     // w^H w
      wn[j] = ww > 0.0 ? 2.0 / ww : 0.0;
      x[j] = wj;
      lgs += log(nrm);             // R_jj = -ph * nrm
      phs = phs * (-cvt<cd>(ph));
    }
    __syncthreads();
    // trailing columns c > j: A[:,c] -= (2/ww) w (w^H A[:,c])
    reflect_columns(N, j + 1, n, j, x, wn[j], Y, warp, nw, lane);
    __syncthreads();
  }
  // Q = H_0 H_1 ... H_{n-1} [I; 0]
  for (int e = tid; e < N * n; e += nt) {
    const int i = e % N, c = e / N;
    Q[e] = i == c ? one<T>() : zero<T>();
  }
  __syncthreads();
  for (int j = n - 1; j >= 0; --j) {
    const T* x = Y + (size_t)j * N;
    reflect_columns(N, j, n, j, x, wn[j], Q, warp, nw, lane);
    __syncthreads();
  }
  if (tid == 0) {
    if (log_out) *log_out = lgs;
    if (phase_out) *phase_out = phs;
  }
}

// ------------------------------------------------------- Cholesky QR (thin Q)
// W = R^H R for the n x n Hermitian positive definite W (ld n), in place: R
// in the upper triangle (real positive diagonal), the strictly lower part
// left as it was.  Sets *bad when a pivot falls to <= tol times the largest
// diagonal entry (W too ill-conditioned for the caller's purpose).  When
// given, log_out receives sum_k log R_kk.  rinv (n entries, shared memory)
// receives 1 / R_kk.
template <class T>
__device__ void chol_upper(int n, T* W, double tol, double* rinv, int* bad, double* log_out = nullptr) {
  const int tid = threadIdx.x, nt = blockDim.x;
  __shared__ double dmax;
  __shared__ double s_r[GJ_DEFER_MAX];   // R_kk, logged after the loop (as in gj_inverse)
  const bool defer = log_out && n <= GJ_DEFER_MAX;
  if (tid == 0) {
    double m = 0.0;
    for (int k = 0; k < n; ++k) m = fmax(m, re(W[k + (size_t)k * n]));
    dmax = m;
  }
  __syncthreads();
  double lgs = 0.0;   // thread 0
  for (int k = 0; k < n; ++k) {
    if (tid == 0) {
      double d = re(W[k + (size_t)k * n]);
      if (!(d > tol * dmax)) {
        *bad = 1;
        d = dmax > 0.0 ? dmax : 1.0;   // keep the arithmetic finite; the caller discards the result
      }
      const double r = sqrt(d);
      W[k + (size_t)k * n] = from_real<T>(r);
      rinv[k] = 1.0 / r;
      if (defer)
        s_r[k] = r;
      else if (log_out)
        lgs += log(r);
    }
    __syncthreads();
    const double s = rinv[k];
    for (int c = k + 1 + tid; c < n; c += nt) W[k + (size_t)c * n] = W[k + (size_t)c * n] * s;   // row k of R
    __syncthreads();
    const int m = n - k - 1;
    for (int e = tid; e < m * m; e += nt) {   // W[i,j] -= conj(R[k,i]) R[k,j], i, j > k
      const int i = k + 1 + e % m, j = k + 1 + e / m;
      W[i + (size_t)j * n] = W[i + (size_t)j * n] - conjg(W[k + (size_t)i * n]) * W[k + (size_t)j * n];
    }
    __syncthreads();
  }
  if (defer) {
    for (int k = tid; k < n; k += nt) s_r[k] = log(s_r[k]);
    __syncthreads();
    if (tid == 0)
      for (int k = 0; k < n; ++k) lgs += s_r[k];
  }
  if (tid == 0 && log_out) *log_out = lgs;
}

// Q (N x n, ld N) = A R^-1 with R upper triangular (ld n, from chol_upper) and
// rinv = 1 / diag(R): one thread per row, forward substitution along the
// columns.  Q must not alias A.
template <class T>
__device__ void trsm_right_upper(int N, int n, const T* A, const T* R, const double* rinv, T* Q) {
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    for (int c = 0; c < n; ++c) {
      T acc = A[i + (size_t)c * N];
      for (int k = 0; k < c; ++k) madd(acc, -Q[i + (size_t)k * N], R[k + (size_t)c * n]);
      Q[i + (size_t)c * N] = normalise(acc) * rinv[c];
    }
  }
  __syncthreads();
}

// --------------------------------------------------------- LU and solves
// In-place LU with partial pivoting of the n x n matrix M (ld n); piv[j]
// receives the row swapped with j (the ?getrf convention).  Returns false
// through *bad when a zero pivot is met.
template <class T>
__device__ void lu_factor(int n, T* M, int* piv, int* bad) {
  const int tid = threadIdx.x, nt = blockDim.x;
  __shared__ int sp;
  for (int j = 0; j < n; ++j) {
    if (tid < 32) {
      double best = -1.0;
      int bi = j;
      for (int i = j + tid; i < n; i += 32) {
        double v = abs2(M[i + (size_t)j * n]);
        if (v > best) { best = v; bi = i; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        double ob = __shfl_xor_sync(0xffffffffu, best, o);
        int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tid == 0) {
        sp = bi;
        piv[j] = bi;
        if (!(best > 0.0)) *bad = 1;
      }
    }
    __syncthreads();
    const int p = sp;
    if (p != j)
      for (int c = tid; c < n; c += nt) {
        T t = M[j + (size_t)c * n];
        M[j + (size_t)c * n] = M[p + (size_t)c * n];
        M[p + (size_t)c * n] = t;
      }
    __syncthreads();
    const T d = M[j + (size_t)j * n];
    for (int i = j + 1 + tid; i < n; i += nt) M[i + (size_t)j * n] = M[i + (size_t)j * n] / d;
    __syncthreads();
    const int m = n - j - 1;
    for (int e = tid; e < m * m; e += nt) {
      const int i = j + 1 + e % m, c = j + 1 + e / m;
      M[i + (size_t)c * n] = M[i + (size_t)c * n] - M[i + (size_t)j * n] * M[j + (size_t)c * n];
    }
    __syncthreads();
  }
}

// In-place inverse of the n x n matrix M (ld n) by Gauss-Jordan elimination
// with partial (row) pivoting; every elimination step is one parallel
// rank-1 update of M, so the inverse costs n^3 multiply-adds at block-GEMM
// parallelism.  f (n elements of shared memory) stages the pivot column;
// cols (n ints) records the row swaps.  *bad is set on a zero pivot.  When
// given, log_out and phase_out receive log|det M| and det M / |det M|.
template <class T>
__device__ void gj_inverse(int n, T* M, T* f, int* swaps, int* bad, double* log_out = nullptr,
                           cd* phase_out = nullptr) {
  const int tid = threadIdx.x, nt = blockDim.x;
  __shared__ int sp;
  __shared__ T s_inv;                // 1 / pivot of the current step
  __shared__ cd s_pv[GJ_DEFER_MAX];  // the pivots, for the determinant after the loop
  __shared__ double s_lg[GJ_DEFER_MAX];
  // the determinant's log and phase are formed after the elimination (each
  // pivot's log and phase in parallel, summed and multiplied in pivot order
  // by thread 0, the same operations in the same order as inside the loop),
  // keeping the FP64 logarithm and quotients off the steps' serial path
  const bool want = log_out || phase_out;
  const bool defer = n <= GJ_DEFER_MAX;
  double lgs = 0.0;          // log |det M| (thread 0)
  cd phs = mkc(1.0, 0.0);    // det M / |det M| (thread 0)
  for (int k = 0; k < n; ++k) {
    if (tid < 32) {
      double best = -1.0;
      int bi = k;
      for (int i = k + tid; i < n; i += 32) {
        const double v = abs2(M[i + (size_t)k * n]);
        if (v > best) { best = v; bi = i; }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (tid == 0) {
        sp = bi;
        swaps[k] = bi;
        if (!(best > 0.0)) *bad = 1;
      }
    }
    __syncthreads();
    const int p = sp;
    if (p != k)
      for (int c = tid; c < n; c += nt) {
        const T tmp = M[k + (size_t)c * n];
        M[k + (size_t)c * n] = M[p + (size_t)c * n];
        M[p + (size_t)c * n] = tmp;
      }
    __syncthreads();
    // scale the pivot row: M[k,k] <- 1, row k <- row k / pivot
    if (tid == 0) {    // det M = (-1)^(row swaps) * product of the pivots
      const T pk = M[k + (size_t)k * n];
      s_inv = one<T>() / pk;
      const cd pv = cvt<cd>(pk);
      if (defer) {
        s_pv[k] = pv;
      } else if (want) {
        const double a = sqrt(abs2(pv));
        lgs += log(a);
        phs = phs * (a > 0.0 ? pv / a : mkc(1.0, 0.0));
        if (p != k) phs = -phs;
      }
    }
    __syncthreads();   // the pivot is read before row k changes
    const T inv = s_inv;
    for (int c = tid; c < n; c += nt) {
      const T v = c == k ? one<T>() : M[k + (size_t)c * n];
      M[k + (size_t)c * n] = v * inv;
    }
    for (int i = tid; i < n; i += nt) f[i] = i == k ? zero<T>() : M[i + (size_t)k * n];
    __syncthreads();
    // eliminate column k from every other row: M[i,:] -= f_i M[k,:] (M[i,k] <- -f_i / pivot)
    for (int e = tid; e < n * n; e += nt) {
      const int i = e % n, c = e / n;
      if (i == k) continue;
      const T base = c == k ? zero<T>() : M[e];
      M[e] = base - f[i] * M[k + (size_t)c * n];
    }
    __syncthreads();
  }
  // undo the row swaps as column swaps, last first
  for (int k = n - 1; k >= 0; --k) {
    const int p = swaps[k];
    if (p != k)
      for (int r = tid; r < n; r += nt) {
        const T tmp = M[r + (size_t)k * n];
        M[r + (size_t)k * n] = M[r + (size_t)p * n];
        M[r + (size_t)p * n] = tmp;
      }
    __syncthreads();
  }
  if (want && defer) {
    for (int k = tid; k < n; k += nt) {
      const cd pv = s_pv[k];
      const double a = sqrt(abs2(pv));
      s_lg[k] = log(a);
      s_pv[k] = a > 0.0 ? pv / a : mkc(1.0, 0.0);
    }
    __syncthreads();
    if (tid == 0)
      for (int k = 0; k < n; ++k) {
        lgs += s_lg[k];
        phs = phs * s_pv[k];
        if (swaps[k] != k) phs = -phs;
      }
  }
  if (tid == 0) {
    if (log_out) *log_out = lgs;
    if (phase_out) *phase_out = phs;
  }
}

// X (n x N, ld n) <- M^{-1} X using the LU factors of lu_factor (?getrs).
// Each thread solves whole columns, so no synchronisation is needed inside.
template <class T>
__device__ void lu_solve(int n, int N, const T* M, const int* piv, T* X) {
  for (int c = threadIdx.x; c < N; c += blockDim.x) {
    T* x = X + (size_t)c * n;
    for (int j = 0; j < n; ++j) {
      const int p = piv[j];
      if (p != j) { T t = x[j]; x[j] = x[p]; x[p] = t; }
    }
    for (int j = 0; j < n; ++j) {
      const T v = x[j];
      for (int i = j + 1; i < n; ++i) x[i] = x[i] - M[i + (size_t)j * n] * v;
    }
    for (int j = n - 1; j >= 0; --j) {
      const T v = x[j] / M[j + (size_t)j * n];
      x[j] = v;
      for (int i = 0; i < j; ++i) x[i] = x[i] - M[i + (size_t)j * n] * v;
    }
  }
  __syncthreads();
}

}  // namespace kdq
