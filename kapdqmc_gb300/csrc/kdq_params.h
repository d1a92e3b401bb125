// Launch parameters and per-chain control words shared by the host runtime
// and the sweep kernels.
#pragma once
#include <cstddef>
#include <cstdint>

#include "../../include/kapdqmc.h"

#define KDQ_MAX_NS 192          // largest lattice (6 row groups of 32 per lane)
#define KDQ_MAX_FIELD 768       // HS fields per slice (t-UV: Ns z with z <= 4)
#define KDQ_MAX_OBS 12          // measurement columns per sweep row
#define KDQ_THREADS 256         // threads per CTA (one CTA per chain)

// device error flags (ChainCtl::err)
#define KDQ_FLAG_NAN 1          // non-finite acceptance ratio
#define KDQ_FLAG_SINGULAR 2     // zero pivot in the G recompute
#define KDQ_FLAG_TAPE 4         // explicit tape exhausted

// KDQ_MODE_SWEEP: every block of one sweep (forward then backward) in one launch
enum { KDQ_MODE_INIT = 0, KDQ_MODE_FWD = 1, KDQ_MODE_BWD = 2, KDQ_MODE_SWEEP = 3 };

struct ChainCtl {
  int idx;              // current stabilisation index (1-based, as the reference)
  int err;              // KDQ_FLAG_* bits
  long long sweep;      // Philox sweep counter
  long long n_prop, n_acc, n_recompute;
  long long tape_pos;   // explicit-tape cursor
  long long log_pos;    // accept-log cursor
  int drift_pos;        // drift-log cursor
  int obs_slot;         // next measurement row of this call
  int obs_cnt;          // measurements accumulated in the current sweep
  int meas_n;           // slice factors held in the fast-measurement products
  double max_drift;
  double obs_acc[KDQ_MAX_OBS];
  // log|det(P^H B(Theta,0) P)| and det/|det| of the fields at the last G recompute
  double logdet, det_re, det_im;
  // self-learning cluster moves of the current call: proposed, accepted,
  // proposals whose effective-model chain changed no site
  long long slmc_prop, slmc_acc, slmc_noop;
};

struct SweepParams {
  // model
  int kind, Ns, Nt, z, n_field, NN, n_obs, record;
  int meas_full;                // t-U, complex t-UV: 4 more columns, the structure factors with all terms
  int lattice, L1, L2;
  int site_nb;                  // tUV: entries per site in site_bonds
  const int64_t* nodes;         // NN
  const double* rtab;           // ratio tables (layout per model, see runtime)
  const double* dtv;            // t-V: per (slice, old, new) the entries of Delta = UV diag(t2) UV:
                                //   d00 (= d11), d01 (= d10), 1 + d00
  const double* dtab;           // tU diagonal tables
  const double* vtab;           // tV exponential tables
  const double* gratio;         // 16: gamma[new]/gamma[old], index old*4+new
  const double* xtab;           // 16: tUV real-type extra weight
  const double* cosr;           // L1*L2 structure-factor phases
  const double* stag;           // Ns: +1 / -1 two-colouring of a bipartite lattice (all 0 if not bipartite)
  const double* eta;            // 4
  double a, Ht, U, V;
  const int* bx;                // 0-based bond ends
  const int* by;
  const int* site_bonds;        // tUV: per site, bond*2 + role (0 first, 1 second), -1 padded
  const void* eK;               // eK, eKinv, HalfeK, HalfeKinv in the working precision
  const void* eKinv;
  const void* HalfeK;
  const void* HalfeKinv;
  // mixed sweep with real kinetic matrices: each of eK, eKinv, HalfeK,
  // HalfeKinv pre-split into TF32 hi/lo words in mma fragment order, as the
  // left (A) and the right (B) operand (kdq_tc.cuh, kin_frag_*), or NULL
  const void* kin_frag;
  size_t kin_frag_words;        // uint4 words per matrix and side
  const void* K;                // FP64
  const void* Pt;
  // chain state (chain-major); G, W1, W2, Yw, Y2w, Lm, Rm are in the working
  // precision, the rest FP64 (in plain mode Yw, Y2w alias Y, Y2 and Gd aliases W1)
  void* G;
  void* W1;
  void* W2;
  void* Y;
  void* Y2;
  void* Yw;
  void* Y2w;
  void* Gd;
  void* Mss;
  void* X;
  void* BLs_;
  void* BRs_;
  int* piv;
  uint8_t* s;
  ChainCtl* ctl;
  size_t sz_NN, sz_Nn, sz_nn, sz_chainB;   // element strides per chain
  // fast measurement (record == 2): L, R products and their factor stack
  void* Lm;
  void* Rm;
  uint8_t* mstack;              // per chain: mstack_max ints (signed slices) + mstack_max field snapshots
  size_t mstack_stride;
  int mstack_max;
  // random stream
  uint64_t seed;
  const uint8_t* tape_k;
  const double* tape_u;
  size_t tape_len;
  // outputs
  double* obs;                  // chain-major rows of n_obs
  int obs_cap;                  // rows per chain
  uint8_t* acc_log;
  long long acc_log_cap;
  double* drift;
  int drift_cap;
  unsigned long long* phase;    // optional per-chain phase clocks (8 per chain), or NULL
  void* gmid;                   // optional per-chain FP64 G at tau = Nt/2 (N x N), or NULL
  // per chain, per node k (1-based) and side (0: BLs, 1: BRs): log|det| and det/|det|
  // of the triangular factors dropped from that side's chain, at
  // lw[((side * NN) + k - 1) * 3 + {0, 1, 2}] (log, re, im)
  double* lw;
  // self-learning cluster moves (t-U): per slice visit, slmc_moves moves of
  // slmc_steps effective-model Metropolis steps on slmc_len consecutive sites;
  // slmc_prm holds the effective model's bf16 weights; the move's shared
  // memory starts slmc_off bytes into the dynamic shared memory
  int slmc_moves, slmc_len, slmc_steps;
  size_t slmc_off;
  const void* slmc_prm;
  // coupled SCEE sweep (t-U): per chain G0, Gt0, G0t (N x N) and the block
  // products BMs, BMi ((NN-1) x N x N); per pair the inverse Grover matrices
  // of regions A and B (scee_nmax^2 each), |det g_A|^2, |det g_B|^2 and the
  // estimator's running sum and count (4 doubles), and scee_O_cap rows
  void* scee_G0;
  void* scee_Gt0;
  void* scee_G0t;
  void* scee_BMs;
  void* scee_BMi;
  void* scee_inv;
  const int* scee_idxA;         // 0-based sites
  const int* scee_idxB;
  int scee_nA, scee_nB, scee_nmax, scee_nlam;
  double scee_lam;
  int scee_dop;                 // 1: disorder-operator sweep of single chains (ctrl_SCDOPicr)
  double scee_alpha;            // its angle
  double* scee_det;
  double* scee_O;
  int scee_O_cap;

  template <class T> __host__ __device__ T* BLs(int c) const { return static_cast<T*>(BLs_) + (size_t)c * sz_chainB; }
  template <class T> __host__ __device__ T* BRs(int c) const { return static_cast<T*>(BRs_) + (size_t)c * sz_chainB; }
};

#ifndef __CUDACC__
#define __host__
#define __device__
#endif
