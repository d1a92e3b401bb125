// Swap-replica Rényi-2 Grover determinant, one CTA per replica pair:
//   g_A = 2 G1_A G2_A - G1_A - G2_A + I   (GroverMatrix!, src/public/GF.jl:101-109)
//   det g_A by LU with partial pivoting  (det in get_ABGM!, src/tU/SCEE.jl:264-276)
// G1_A, G2_A are the region-A blocks of the two replicas' equal-time Green's
// functions.  Scratch per pair: the two gathered blocks and g_A (3 nA^2
// elements) plus nA pivots.
#pragma once
#include "kdq_device.cuh"

namespace kdq {

template <class T>
__device__ void grover_pair(const T* G1, const T* G2, int Ns, const int* index, int nA, T* A, T* B,
                            T* gm, int* piv, double* det_out) {
  const int n2 = nA * nA;
  for (int e = threadIdx.x; e < n2; e += blockDim.x) {
    const int i = e % nA, j = e / nA;
    const size_t src = (size_t)index[i] + (size_t)index[j] * Ns;
    A[e] = G1[src];
    B[e] = G2[src];
  }
  __syncthreads();
  bgemm_t<2, 4>(nA, nA, nA, A, nA, B, nA, gm, nA);
  for (int e = threadIdx.x; e < n2; e += blockDim.x) {
    const int i = e % nA, j = e / nA;
    T v = (gm[e] * 2.0 - A[e]) - B[e];
    if (i == j) v = v + one<T>();
    gm[e] = v;
  }
  __syncthreads();
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  lu_factor(nA, gm, piv, &bad);
  if (threadIdx.x == 0) {
    T d = one<T>();
    int swaps = 0;
    for (int j = 0; j < nA; ++j) {
      d = d * gm[j + (size_t)j * nA];
      swaps += piv[j] != j;
    }
    if (swaps & 1) d = zero<T>() - d;
    if constexpr (sizeof(T) == sizeof(cd)) {
      det_out[0] = reinterpret_cast<const cd&>(d).x;
      det_out[1] = reinterpret_cast<const cd&>(d).y;
    } else {
      det_out[0] = re(d);
      det_out[1] = 0.0;
    }
  }
}

// G: 2*npairs matrices of Ns x Ns (pair p = matrices 2p, 2p+1), stride
// Ns*Ns elements; index: nA 0-based sites; det: 2 doubles per pair.
template <class T>
__global__ void __launch_bounds__(256) k_grover(const T* G, int Ns, const int* index, int nA, int npairs,
                                                T* scratch, int* pivs, double* det) {
  const int p = blockIdx.x;
  if (p >= npairs) return;
  const size_t NN = (size_t)Ns * Ns, n2 = (size_t)nA * nA;
  T* A = scratch + (size_t)p * 3 * n2;
  grover_pair(G + 2 * p * NN, G + (2 * p + 1) * NN, Ns, index, nA, A, A + n2, A + 2 * n2,
              pivs + (size_t)p * nA, det + 2 * p);
}

}  // namespace kdq
