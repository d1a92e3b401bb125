// Host runtime of libkapdqmc_gpu.so: handle lifecycle, model upload,
// precomputed slice tables, launch sequencing of the sweep, and the C ABI
// declared in include/kapdqmc.h.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "kdq_cnn.cuh"
#include "kdq_launch.h"
#include "kdq_params.h"
#include "kdq_tc.cuh"

using cplx = std::complex<double>;

namespace {

std::mutex g_err_mu;
std::string g_create_err;

// tile classes chosen by kdq_autotune, per device, model, size, precision
// and batch (process-wide, so later handles of the same shape reuse them)
struct TuneKey {
  int device, kind, Ns, Nt;
  bool gc, kc;
  int precision, nchains, slmc;
  bool operator==(const TuneKey& o) const {
    return device == o.device && kind == o.kind && Ns == o.Ns && Nt == o.Nt && gc == o.gc && kc == o.kc &&
           precision == o.precision && nchains == o.nchains && slmc == o.slmc;
  }
};
struct TuneEntry {
  TuneKey key;
  int rows;
  double ms[3];
};
std::mutex g_tune_mu;
std::vector<TuneEntry> g_tune;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  cudaError_t alloc(size_t b) {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    if (b == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, b);
    if (e == cudaSuccess) bytes = b;
    return e;
  }
  template <class T> T* as() const { return static_cast<T*>(p); }
};

}  // namespace

struct kdq_handle {
  int device = 0;
  int nchains = 0;
  int kind = 0, Ns = 0, ns = 0, Nt = 0, z = 1, n_field = 0, NN = 0, n_obs = 0;
  bool gc = true, kc = false;
  int maxrm = 1;
  size_t esz = 16;   // bytes per G element
  size_t dyn = 0;    // dynamic shared memory per CTA
  size_t dyn_base = 0;   // the tape slice's part of it
  cudaStream_t stream = nullptr;
  std::string err;
  SweepParams P{};
  // model buffers
  DevBuf nodes, rtab, dtab, vtab, gratio, xtab, cosr, stag, eta, bx, by, site_bonds, dtv;
  DevBuf eK, eKinv, HalfeK, HalfeKinv, K, Pt, PtH;
  // chain buffers
  DevBuf G, W1, W2, Y, Y2, Mss, X, piv, BLs, BRs, s, ctl;
  DevBuf Lm, Rm, mstack;   // fast-measurement products, allocated on first use
  // mixed precision: FP32 working buffers and kinetic matrices, FP64 recompute product
  int precision = KDQ_PREC_FP64;
  size_t esz_w = 16;       // bytes per working-precision G element
  DevBuf Yw, Y2w, Gd, eKw, eKinvw, HalfeKw, HalfeKinvw;
  DevBuf kinfrag;     // mixed, real kinetic matrices: the pre-split tensor-core operands
  DevBuf Pts, PtHs;   // mixed: Pt and Pt^H in the double-float stabilisation type
  DevBuf phase;            // per-chain phase clocks when enabled
  DevBuf gmid;             // per-chain G at tau = Nt/2 when enabled
  DevBuf lw;               // per-chain log|det| of the dropped QR factors per node
  DevBuf slmc_prm;         // effective-model weights (bf16) of the cluster moves
  // coupled SCEE sweep buffers (kdq_scee_enable)
  DevBuf scee_G0, scee_Gt0, scee_G0t, scee_BMs, scee_BMi, scee_inv, scee_idx, scee_det, scee_O;
  bool scee = false;
  double scee_lam = 0.0;
  // outputs
  DevBuf obs, acc_log, drift, tape_k, tape_u;
  // Grover-determinant workspace
  DevBuf gr_scratch, gr_piv, gr_index, gr_det;
  int obs_rows = 0;      // rows recorded since kdq_init
  int obs_capacity = 0;  // rows allocated
  long long acc_log_cap = 0;
  int drift_cap = 0;
  uint64_t seed = 0;
  bool use_tape = false;
  size_t tape_len = 0;
  double last_seconds = 0.0;
  bool initialised = false;
  int drift_rows = 0;           // drift entries per chain written by the last call
  // one sweep (2 (NN-1) block launches) captured as a CUDA graph, replayed
  // while the launch parameters stay the same
  bool use_graphs = true;
  bool sweep_launch = false;  // one launch per sweep (else, the default, one per stabilisation block)
  cudaGraphExec_t graph = nullptr;
  SweepParams graph_P{};
  ~kdq_handle() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

namespace {

int fail(kdq_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

int cuda_fail(kdq_handle* h, cudaError_t e, const char* what) {
  return fail(h, KDQ_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define KDQ_CUDA(h, call)                                    \
  do {                                                       \
    cudaError_t _e = (call);                                 \
    if (_e != cudaSuccess) return cuda_fail((h), _e, #call); \
  } while (0)

template <class V>
cudaError_t upload(DevBuf& b, const V& v) {
  cudaError_t e = b.alloc(v.size() * sizeof(v[0]));
  if (e != cudaSuccess || v.empty()) return e;
  return cudaMemcpy(b.p, v.data(), v.size() * sizeof(v[0]), cudaMemcpyHostToDevice);
}

// Model matrices as delivered: n x m, complex interleaved iff cplx_in; stored
// on the device as complex (to_c) or real.
cudaError_t upload_mat(DevBuf& b, const double* src, size_t n, bool cplx_in, bool to_c) {
  std::vector<double> v(n * (to_c ? 2 : 1));
  for (size_t i = 0; i < n; ++i) {
    const double re = cplx_in ? src[2 * i] : src[i];
    const double im = cplx_in ? src[2 * i + 1] : 0.0;
    if (to_c) {
      v[2 * i] = re;
      v[2 * i + 1] = im;
    } else {
      v[i] = re;
    }
  }
  return upload(b, v);
}

// Launch one stabilisation block for all chains.
cudaError_t launch(kdq_handle* h, int mode, int k) {
  if (h->precision == KDQ_PREC_MIXED) {
    // the tensor-core kinetic products read the pre-split operands
    if (!h->kc && !h->P.kin_frag) return cudaErrorInvalidValue;
    switch (h->kind) {
      case KDQ_TU:
        return kdq::launch_tu_mixed(h->P, mode, k, h->maxrm, h->kc, h->nchains, h->dyn, h->stream);
      case KDQ_TV:
        return kdq::launch_tv_mixed(h->P, mode, k, h->maxrm, h->nchains, h->dyn, h->stream);
      default:
        return kdq::launch_tuv_mixed(h->P, mode, k, h->maxrm, h->gc, h->nchains, h->dyn, h->stream);
    }
  }
  switch (h->kind) {
    case KDQ_TU:
      return kdq::launch_tu(h->P, mode, k, h->maxrm, h->kc, h->nchains, h->dyn, h->stream);
    case KDQ_TV:
      return kdq::launch_tv(h->P, mode, k, h->maxrm, h->nchains, h->dyn, h->stream);
    default:
      return kdq::launch_tuv(h->P, mode, k, h->maxrm, h->gc, h->nchains, h->dyn, h->stream);
  }
}

__global__ void k_seed_chains(void* BRs, void* BLs, const void* Pt, const void* PtH, size_t fs,
                              size_t chainB, int NN, size_t esz, double* lw) {
  // BRs[1] = Pt, BLs[NN] = Pt^H for chain blockIdx.x (byte copies); no
  // factor has been dropped from either end yet (log 0, phase 1)
  if (threadIdx.x < 2) {
    double* w = lw + ((size_t)blockIdx.x * 2 * NN + (threadIdx.x == 0 ? NN - 1 : NN)) * 3;
    w[0] = 0.0;
    w[1] = 1.0;
    w[2] = 0.0;
  }
  const size_t bytes = fs * esz;
  uint8_t* br = static_cast<uint8_t*>(BRs) + (size_t)blockIdx.x * chainB * esz;
  uint8_t* bl = static_cast<uint8_t*>(BLs) + ((size_t)blockIdx.x * chainB + (size_t)(NN - 1) * fs) * esz;
  const uint8_t* pt = static_cast<const uint8_t*>(Pt);
  const uint8_t* ph = static_cast<const uint8_t*>(PtH);
  for (size_t i = threadIdx.x; i < bytes; i += blockDim.x) {
    br[i] = pt[i];
    bl[i] = ph[i];
  }
}

// FP64 -> double-float pairs (hi, lo): the mixed sweep's stabilisation type
__global__ void k_to_dfl(const double* src, float* dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double v = src[i];
    const float hi = __double2float_rn(v);
    dst[2 * i] = hi;
    dst[2 * i + 1] = __double2float_rn(v - (double)hi);
  }
}

// The TF32 hi/lo fragment layouts of one real N x N kinetic matrix as the
// left and the right tensor-core operand (kin_frag_word, kdq_tc.cuh).
__global__ void k_kin_frag(const float* kin, int N, uint4* left, uint4* right) {
  const size_t k8 = (N + 7) / 8, m16 = (N + 15) / 16;
  const size_t n = (m16 > k8 ? m16 : k8) * k8 * 32;
  for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x)
    kdq::kin_frag_word(kin, N, e, left, right);
}

__global__ void k_to_float(const double* src, float* dst, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

__global__ void k_reset_ctl(ChainCtl* ctl, int n, int full) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  ChainCtl& x = ctl[c];
  if (full) {
    x.idx = 1;
    x.obs_slot = 0;
    x.obs_cnt = 0;
    x.meas_n = 0;
    for (int q = 0; q < KDQ_MAX_OBS; ++q) x.obs_acc[q] = 0.0;
  }
  x.err = 0;
  x.n_prop = x.n_acc = x.n_recompute = 0;
  x.log_pos = 0;
  x.drift_pos = 0;
  x.max_drift = 0.0;
  x.slmc_prop = x.slmc_acc = x.slmc_noop = 0;
}

__global__ void k_set_sweep(ChainCtl* ctl, int n, long long sweep, int reset_tape) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  ctl[c].sweep = sweep;
  if (reset_tape) ctl[c].tape_pos = 0;
}

int validate(const kdq_model_desc* m, int nchains, std::string& why) {
  if (!m) { why = "model is NULL"; return 1; }
  if (m->kind < KDQ_TU || m->kind > KDQ_TUV) { why = "unknown model kind"; return 1; }
  if (m->Ns < 2 || (m->Ns & 1) || m->Ns > KDQ_MAX_NS) {
    why = "Ns must be even and in [2, " + std::to_string(KDQ_MAX_NS) + "]";
    return 1;
  }
  if (m->Nt < 1 || m->n_nodes < 2 || !m->nodes) { why = "need Nt >= 1 and >= 2 nodes"; return 1; }
  if (m->nodes[0] != 0 || m->nodes[m->n_nodes - 1] != m->Nt) { why = "nodes must run from 0 to Nt"; return 1; }
  for (int i = 1; i < m->n_nodes; ++i)
    if (m->nodes[i] <= m->nodes[i - 1]) { why = "nodes must increase strictly"; return 1; }
  if (nchains < 1) { why = "n_chains must be >= 1"; return 1; }
  if (!m->eK || !m->eKinv || !m->HalfeK || !m->HalfeKinv || !m->K || !m->Pt || !m->gamma || !m->eta) {
    why = "missing model array";
    return 1;
  }
  if (m->kind != KDQ_TUV && !m->alpha) { why = "alpha is required for tU and tV"; return 1; }
  if (m->kind != KDQ_TU && (!m->bonds || m->z < 1)) { why = "bonds and z are required for tV and tUV"; return 1; }
  if (m->kind == KDQ_TU && !m->g_complex) { why = "the tU sweep is complex"; return 1; }
  if (m->kind == KDQ_TV && (m->g_complex || m->k_complex)) { why = "the tV sweep is real"; return 1; }
  if (m->kind == KDQ_TUV && m->k_complex) { why = "tUV kinetic matrices are real"; return 1; }
  const int nb = m->kind == KDQ_TV ? (m->Ns / 2) * m->z : m->Ns * m->z;
  if (m->kind != KDQ_TU && nb > KDQ_MAX_FIELD) {
    why = "too many bonds per slice (at most " + std::to_string(KDQ_MAX_FIELD) + ")";
    return 1;
  }
  if (m->kind != KDQ_TU)
    for (int b = 0; b < 2 * nb; ++b)
      if (m->bonds[b] < 1 || m->bonds[b] > m->Ns) { why = "bond index out of range"; return 1; }
  if (m->kind == KDQ_TV) {
    // every direction must be a perfect matching (the 2x2 block rotations
    // rely on it; src/tV/model.jl:103-110 builds UV from such bonds)
    std::vector<int> seen(m->Ns);
    for (int j = 0; j < m->z; ++j) {
      std::fill(seen.begin(), seen.end(), 0);
      for (int i = 0; i < m->Ns / 2; ++i) {
        const int* bnd = m->bonds + 2 * (j * (m->Ns / 2) + i);
        if (seen[bnd[0] - 1]++ || seen[bnd[1] - 1]++) { why = "tV bond direction is not a perfect matching"; return 1; }
      }
    }
  }
  const bool hc = m->lattice == KDQ_HONEYCOMB120 || m->lattice == KDQ_HONEYCOMB60;
  if (hc && 2 * m->site[0] * m->site[1] != m->Ns) { why = "site does not match Ns"; return 1; }
  return 0;
}

}  // namespace

extern "C" {

const char* kdq_last_error(const kdq_handle* h) {
  if (h) return h->err.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_create_err.c_str();
}

void kdq_destroy(kdq_handle* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

void* kdq_stream(kdq_handle* h) { return h ? (void*)h->stream : nullptr; }

int kdq_n_obs(const kdq_handle* h) { return h ? h->n_obs : 0; }

int kdq_create(kdq_handle** out, const kdq_model_desc* m, int32_t nchains, int32_t device) {
  auto set_err = [](int code, const std::string& msg) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_err = msg;
    return code;
  };
  if (!out) return set_err(KDQ_ERR_ARG, "out is NULL");
  *out = nullptr;
  std::string why;
  if (validate(m, nchains, why)) return set_err(KDQ_ERR_ARG, why);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return set_err(KDQ_ERR_NOGPU, "no CUDA device");
  if (device < 0 || device >= ndev) return set_err(KDQ_ERR_ARG, "device out of range");
  cudaError_t ce = cudaSetDevice(device);
  if (ce != cudaSuccess) return set_err(KDQ_ERR_CUDA, cudaGetErrorString(ce));

  kdq_handle* h = new kdq_handle();
  h->device = device;
  h->nchains = nchains;
  h->kind = m->kind;
  h->Ns = m->Ns;
  h->ns = m->Ns / 2;
  h->Nt = m->Nt;
  h->z = m->kind == KDQ_TU ? 1 : m->z;
  h->NN = m->n_nodes;
  h->gc = m->g_complex != 0;
  h->kc = m->k_complex != 0;
  h->esz = h->gc ? 16 : 8;
  h->esz_w = h->esz;
  h->n_field = m->kind == KDQ_TU ? m->Ns : (m->kind == KDQ_TV ? (m->Ns / 2) * h->z : m->Ns * h->z);
  h->n_obs = m->kind == KDQ_TU ? 6 : (m->kind == KDQ_TV ? 10 : 7);
  h->maxrm = m->Ns <= 32 ? 1 : (m->Ns <= 96 ? 3 : 6);
  h->dyn = ((size_t)h->n_field * 9 + 15) & ~(size_t)15;
  h->dyn_base = h->dyn;
  auto bail = [&](int code) {
    int rc = set_err(code, h->err);
    kdq_destroy(h);
    return rc;
  };
#define KDQ_CK(call)                                 \
  do {                                               \
    cudaError_t _e = (call);                         \
    if (_e != cudaSuccess) {                         \
      cuda_fail(h, _e, #call);                       \
      return bail(KDQ_ERR_CUDA);                     \
    }                                                \
  } while (0)
  KDQ_CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));

  const int N = h->Ns, ns = h->ns, Nt = h->Nt;
  const double* g = m->gamma;
  const double* eta = m->eta;
  // ---- tables
  std::vector<double> gr(16), xt(16, 1.0);
  for (int o = 0; o < 4; ++o)
    for (int v = 0; v < 4; ++v) gr[o * 4 + v] = g[v] / g[o];
  std::vector<int64_t> nodes(m->nodes, m->nodes + m->n_nodes);
  KDQ_CK(upload(h->nodes, nodes));
  KDQ_CK(upload(h->gratio, gr));
  KDQ_CK(upload(h->eta, std::vector<double>(eta, eta + 4)));
  if (m->kind == KDQ_TU) {
    // D = cis(α η), 1 ./ D, cis(-α η), 1 ./ cis(-α η)  (src/tU/phy_update.jl:61-63,123-125)
    std::vector<double> dt((size_t)Nt * 16 * 2), rt((size_t)Nt * 16 * 2);
    for (int lt = 0; lt < Nt; ++lt) {
      const double al = m->alpha[lt];
      for (int v = 0; v < 4; ++v) {
        const cplx dp = std::polar(1.0, al * eta[v]);
        const cplx dm = std::polar(1.0, -al * eta[v]);
        const cplx e4[4] = {dp, 1.0 / dp, dm, 1.0 / dm};
        for (int q = 0; q < 4; ++q) {
          dt[((size_t)lt * 16 + q * 4 + v) * 2] = e4[q].real();
          dt[((size_t)lt * 16 + q * 4 + v) * 2 + 1] = e4[q].imag();
        }
      }
      // get_r!: Δ = cis(α(η_new - η_old)) - 1  (src/tU/GreenMatrix.jl:49-54)
      for (int o = 0; o < 4; ++o)
        for (int v = 0; v < 4; ++v) {
          const cplx d = std::polar(1.0, al * (eta[v] - eta[o])) - 1.0;
          rt[((size_t)lt * 16 + o * 4 + v) * 2] = d.real();
          rt[((size_t)lt * 16 + o * 4 + v) * 2 + 1] = d.imag();
        }
    }
    KDQ_CK(upload(h->dtab, dt));
    KDQ_CK(upload(h->rtab, rt));
  } else if (m->kind == KDQ_TV) {
    // bond exponentials (src/tV/phy_update.jl:64-71,133-138) and
    // Δ entries exp(±Δs) - 1 (src/tV/GreenMatrix.jl:76-78)
    std::vector<double> vt((size_t)Nt * 32), rt((size_t)Nt * 16 * 2);
    for (int lt = 0; lt < Nt; ++lt) {
      const double al = m->alpha[lt];
      for (int v = 0; v < 4; ++v) {
        const double x = al * eta[v];
        const double fx = std::exp(x), fy = std::exp(-al * eta[v]);
        double* t = vt.data() + (size_t)lt * 32;
        t[v] = fx; t[4 + v] = fy; t[8 + v] = 1.0 / fx; t[12 + v] = 1.0 / fy;
        const double bx_ = std::exp(-x), by_ = std::exp(-(-al * eta[v]));
        t[16 + v] = bx_; t[20 + v] = by_; t[24 + v] = 1.0 / bx_; t[28 + v] = 1.0 / by_;
      }
      for (int o = 0; o < 4; ++o)
        for (int v = 0; v < 4; ++v) {
          const double ds = al * (eta[v] - eta[o]);
          rt[((size_t)lt * 16 + o * 4 + v) * 2] = std::exp(ds) - 1.0;
          rt[((size_t)lt * 16 + o * 4 + v) * 2 + 1] = std::exp(-ds) - 1.0;
        }
    }
    // the entries of Δ = uv diag(t2) uv (uv = [-h -h; -h h]) and 1 + Δ_00 per
    // (slice, old, new), for the acceptance ratio
    std::vector<double> dv((size_t)Nt * 16 * 3);
    const double hh = 0.70710678118654752440;
    for (size_t q = 0; q < (size_t)Nt * 16; ++q) {
      const double t0 = rt[2 * q], t1 = rt[2 * q + 1];
      const double dd = std::fma(-hh * t0, -hh, (-hh * t1) * -hh);
      const double dof = std::fma(-hh * t0, -hh, (-hh * t1) * hh);
      dv[3 * q] = dd;
      dv[3 * q + 1] = dof;
      dv[3 * q + 2] = 1.0 + dd;
    }
    KDQ_CK(upload(h->vtab, vt));
    KDQ_CK(upload(h->rtab, rt));
    KDQ_CK(upload(h->dtv, dv));
  } else {
    // Δ = diag(e^{iΔs}-1, e^{iaΔs}-1) or the real exponentials, and the
    // real-type weight exp((η_old-η_new)(a+1))  (src/tUV/GreenMatrix.jl:73-89,
    // src/tUV/phy_update.jl:195-197)
    std::vector<double> rt(16 * 2 * (h->gc ? 2 : 1));
    for (int o = 0; o < 4; ++o)
      for (int v = 0; v < 4; ++v) {
        const double ds = eta[v] - eta[o];
        const double t2[2] = {ds, ds * m->a};
        for (int q = 0; q < 2; ++q) {
          if (h->gc) {
            const cplx d = std::polar(1.0, t2[q]) - 1.0;
            rt[((o * 4 + v) * 2 + q) * 2] = d.real();
            rt[((o * 4 + v) * 2 + q) * 2 + 1] = d.imag();
          } else {
            rt[(o * 4 + v) * 2 + q] = std::exp(t2[q]) - 1.0;
          }
        }
        if (!h->gc) xt[o * 4 + v] = std::exp((eta[o] - eta[v]) * (m->a + 1.0));
      }
    KDQ_CK(upload(h->rtab, rt));
  }
  KDQ_CK(upload(h->xtab, xt));
  // structure-factor phases cos(2π/L1 rx + 2π/L2 ry)
  const int L1 = m->site[0] > 0 ? m->site[0] : 1, L2 = m->site[1] > 0 ? m->site[1] : 1;
  std::vector<double> cr((size_t)L1 * L2);
  for (int ry = 1; ry <= L2; ++ry)
    for (int rx = 1; rx <= L1; ++rx)
      cr[(rx - 1) + (size_t)(ry - 1) * L1] = std::cos(2 * M_PI / L1 * rx + 2 * M_PI / L2 * ry);
  KDQ_CK(upload(h->cosr, cr));
  // two-colouring of the hopping graph (nonzero K entries): the staggered
  // sign of the (pi, pi) structure factors on the square lattices
  {
    std::vector<double> sg(N, 0.0);
    auto kabs = [&](int i, int j) {
      const size_t e = i + (size_t)j * N;
      return h->kc ? std::hypot(m->K[2 * e], m->K[2 * e + 1]) : std::fabs(m->K[e]);
    };
    bool bip = true;
    std::vector<int> stack;
    for (int root = 0; root < N && bip; ++root) {
      if (sg[root] != 0.0) continue;
      sg[root] = 1.0;
      stack.assign(1, root);
      while (!stack.empty() && bip) {
        const int i = stack.back();
        stack.pop_back();
        for (int j = 0; j < N; ++j) {
          if (j == i || !(kabs(i, j) > 1e-12)) continue;
          if (sg[j] == 0.0) {
            sg[j] = -sg[i];
            stack.push_back(j);
          } else if (sg[j] == sg[i]) {
            bip = false;
            break;
          }
        }
      }
    }
    if (!bip) std::fill(sg.begin(), sg.end(), 0.0);
    KDQ_CK(upload(h->stag, sg));
  }
  // bonds (0-based) and the tUV per-site bond lists
  int site_nb = 0;
  if (m->kind != KDQ_TU) {
    const int nb = m->kind == KDQ_TV ? (N / 2) * h->z : N * h->z;
    std::vector<int> bx(nb), by(nb);
    for (int b = 0; b < nb; ++b) {
      bx[b] = m->bonds[2 * b] - 1;
      by[b] = m->bonds[2 * b + 1] - 1;
    }
    KDQ_CK(upload(h->bx, bx));
    KDQ_CK(upload(h->by, by));
    if (m->kind == KDQ_TUV) {
      std::vector<std::vector<int>> lists(N);
      for (int b = 0; b < nb; ++b) {
        lists[bx[b]].push_back(2 * b);
        lists[by[b]].push_back(2 * b + 1);
      }
      for (auto& l : lists) site_nb = std::max<int>(site_nb, (int)l.size());
      std::vector<int> flat((size_t)N * site_nb, -1);
      for (int x = 0; x < N; ++x)
        for (size_t q = 0; q < lists[x].size(); ++q) flat[(size_t)x * site_nb + q] = lists[x][q];
      KDQ_CK(upload(h->site_bonds, flat));
    }
  }
  // ---- model matrices
  const size_t NNe = (size_t)N * N;
  KDQ_CK(upload_mat(h->eK, m->eK, NNe, h->kc, h->kc));
  KDQ_CK(upload_mat(h->eKinv, m->eKinv, NNe, h->kc, h->kc));
  KDQ_CK(upload_mat(h->HalfeK, m->HalfeK, NNe, h->kc, h->kc));
  KDQ_CK(upload_mat(h->HalfeKinv, m->HalfeKinv, NNe, h->kc, h->kc));
  KDQ_CK(upload_mat(h->K, m->K, NNe, h->kc, h->kc));
  KDQ_CK(upload_mat(h->Pt, m->Pt, (size_t)N * ns, h->gc, h->gc));
  {  // Pt^H (ns x N)
    std::vector<double> ph((size_t)N * ns * (h->gc ? 2 : 1));
    for (int i = 0; i < N; ++i)
      for (int c = 0; c < ns; ++c) {
        const size_t src = i + (size_t)c * N, dst = c + (size_t)i * ns;
        if (h->gc) {
          ph[2 * dst] = m->Pt[2 * src];
          ph[2 * dst + 1] = -m->Pt[2 * src + 1];
        } else {
          ph[dst] = m->Pt[src];
        }
      }
    KDQ_CK(upload(h->PtH, ph));
  }
  // ---- chain state
  const size_t C = nchains, e = h->esz;
  const size_t chainB = (size_t)h->NN * N * ns;
  KDQ_CK(h->G.alloc(C * NNe * e));
  KDQ_CK(h->W1.alloc(C * NNe * e));
  KDQ_CK(h->W2.alloc(C * NNe * e));
  KDQ_CK(h->Y.alloc(C * N * ns * e));
  KDQ_CK(h->Y2.alloc(C * N * ns * e));
  KDQ_CK(h->X.alloc(C * N * ns * e));
  KDQ_CK(h->Mss.alloc(C * ns * ns * e));
  KDQ_CK(h->piv.alloc(C * ns * sizeof(int)));
  KDQ_CK(h->BLs.alloc(C * chainB * e));
  KDQ_CK(h->BRs.alloc(C * chainB * e));
  KDQ_CK(h->s.alloc(C * Nt * h->n_field));
  KDQ_CK(h->ctl.alloc(C * sizeof(ChainCtl)));
  KDQ_CK(cudaMemset(h->ctl.p, 0, C * sizeof(ChainCtl)));
  KDQ_CK(h->lw.alloc(C * 6 * (size_t)h->NN * sizeof(double)));
  KDQ_CK(cudaMemset(h->lw.p, 0, C * 6 * (size_t)h->NN * sizeof(double)));
  KDQ_CK(cudaMemset(h->G.p, 0, C * NNe * e));
  KDQ_CK(h->obs.alloc(8));

  SweepParams& P = h->P;
  P.kind = h->kind; P.Ns = N; P.Nt = Nt; P.z = h->z; P.n_field = h->n_field; P.NN = h->NN;
  P.n_obs = h->n_obs; P.record = 0; P.lattice = m->lattice; P.L1 = L1; P.L2 = L2; P.site_nb = site_nb;
  P.nodes = h->nodes.as<int64_t>(); P.rtab = h->rtab.as<double>();
  P.dtv = h->dtv.as<double>(); P.dtab = h->dtab.as<double>();
  P.vtab = h->vtab.as<double>(); P.gratio = h->gratio.as<double>(); P.xtab = h->xtab.as<double>();
  P.cosr = h->cosr.as<double>(); P.stag = h->stag.as<double>(); P.eta = h->eta.as<double>();
  P.a = m->a; P.Ht = m->Ht; P.U = m->U; P.V = m->V;
  P.bx = h->bx.as<int>(); P.by = h->by.as<int>(); P.site_bonds = h->site_bonds.as<int>();
  P.eK = h->eK.p; P.eKinv = h->eKinv.p; P.HalfeK = h->HalfeK.p; P.HalfeKinv = h->HalfeKinv.p;
  P.K = h->K.p; P.Pt = h->Pt.p;
  P.G = h->G.p; P.W1 = h->W1.p; P.W2 = h->W2.p; P.Y = h->Y.p; P.Y2 = h->Y2.p; P.Mss = h->Mss.p;
  P.Yw = h->Y.p; P.Y2w = h->Y2.p; P.Gd = h->W1.p;
  P.X = h->X.p; P.BLs_ = h->BLs.p; P.BRs_ = h->BRs.p; P.piv = h->piv.as<int>();
  P.s = h->s.as<uint8_t>(); P.ctl = h->ctl.as<ChainCtl>(); P.lw = h->lw.as<double>();
  P.sz_NN = NNe; P.sz_Nn = (size_t)N * ns; P.sz_nn = (size_t)ns * ns; P.sz_chainB = chainB;
  P.seed = 0; P.tape_k = nullptr; P.tape_u = nullptr; P.tape_len = 0;
  P.obs = h->obs.as<double>(); P.obs_cap = 0;
  P.acc_log = nullptr; P.acc_log_cap = 0; P.drift = nullptr; P.drift_cap = 0;
  KDQ_CK(cudaDeviceSynchronize());
#undef KDQ_CK
  *out = h;
  return KDQ_OK;
}

int kdq_set_fields(kdq_handle* h, const uint8_t* s, size_t nbytes) {
  if (!h || !s) return fail(h, KDQ_ERR_ARG, "NULL argument");
  const size_t want = (size_t)h->nchains * h->Nt * h->n_field;
  if (nbytes != want) return fail(h, KDQ_ERR_ARG, "field size mismatch: expected " + std::to_string(want));
  for (size_t i = 0; i < nbytes; ++i)
    if (s[i] < 1 || s[i] > 4) return fail(h, KDQ_ERR_ARG, "HS field values must be in 1..4");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaMemcpyAsync(h->s.p, s, nbytes, cudaMemcpyHostToDevice, h->stream));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  h->initialised = false;
  return KDQ_OK;
}

int kdq_get_fields(kdq_handle* h, uint8_t* s, size_t nbytes) {
  if (!h || !s) return fail(h, KDQ_ERR_ARG, "NULL argument");
  const size_t want = (size_t)h->nchains * h->Nt * h->n_field;
  if (nbytes != want) return fail(h, KDQ_ERR_ARG, "field size mismatch: expected " + std::to_string(want));
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaMemcpyAsync(s, h->s.p, nbytes, cudaMemcpyDeviceToHost, h->stream));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  return KDQ_OK;
}

int kdq_set_rng(kdq_handle* h, uint64_t seed, uint64_t sweep_offset) {
  if (!h) return KDQ_ERR_ARG;
  KDQ_CUDA(h, cudaSetDevice(h->device));
  h->seed = seed;
  h->use_tape = false;
  h->P.seed = seed;
  h->P.tape_k = nullptr;
  h->P.tape_u = nullptr;
  h->P.tape_len = 0;
  k_set_sweep<<<(h->nchains + 127) / 128, 128, 0, h->stream>>>(h->ctl.as<ChainCtl>(), h->nchains,
                                                              (long long)sweep_offset, 1);
  KDQ_CUDA(h, cudaGetLastError());
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  return KDQ_OK;
}

int kdq_set_tape(kdq_handle* h, const uint8_t* k, const double* u, size_t n_per_chain) {
  if (!h || !k || !u) return fail(h, KDQ_ERR_ARG, "NULL argument");
  for (size_t i = 0; i < n_per_chain * h->nchains; ++i) {
    if (k[i] > 2) return fail(h, KDQ_ERR_ARG, "tape choice index must be 0, 1 or 2");
    if (!(u[i] >= 0.0 && u[i] < 1.0)) return fail(h, KDQ_ERR_ARG, "tape uniforms must lie in [0, 1)");
  }
  KDQ_CUDA(h, cudaSetDevice(h->device));
  const size_t n = n_per_chain * h->nchains;
  KDQ_CUDA(h, h->tape_k.alloc(n));
  KDQ_CUDA(h, h->tape_u.alloc(n * sizeof(double)));
  KDQ_CUDA(h, cudaMemcpy(h->tape_k.p, k, n, cudaMemcpyHostToDevice));
  KDQ_CUDA(h, cudaMemcpy(h->tape_u.p, u, n * sizeof(double), cudaMemcpyHostToDevice));
  h->use_tape = true;
  h->tape_len = n_per_chain;
  h->P.tape_k = h->tape_k.as<uint8_t>();
  h->P.tape_u = h->tape_u.as<double>();
  h->P.tape_len = n_per_chain;
  k_set_sweep<<<(h->nchains + 127) / 128, 128, 0, h->stream>>>(h->ctl.as<ChainCtl>(), h->nchains, 0, 1);
  KDQ_CUDA(h, cudaGetLastError());
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  return KDQ_OK;
}

int kdq_enable_accept_log(kdq_handle* h, size_t n_per_chain) {
  if (!h) return KDQ_ERR_ARG;
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, h->acc_log.alloc(n_per_chain * h->nchains));
  if (n_per_chain) KDQ_CUDA(h, cudaMemset(h->acc_log.p, 0xff, n_per_chain * h->nchains));
  h->acc_log_cap = (long long)n_per_chain;
  h->P.acc_log = n_per_chain ? h->acc_log.as<uint8_t>() : nullptr;
  h->P.acc_log_cap = h->acc_log_cap;
  return KDQ_OK;
}

int kdq_get_accept_log(kdq_handle* h, uint8_t* flags, size_t nbytes) {
  if (!h || !flags) return fail(h, KDQ_ERR_ARG, "NULL argument");
  if (nbytes != (size_t)h->acc_log_cap * h->nchains) return fail(h, KDQ_ERR_ARG, "accept-log size mismatch");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  KDQ_CUDA(h, cudaMemcpy(flags, h->acc_log.p, nbytes, cudaMemcpyDeviceToHost));
  return KDQ_OK;
}

int kdq_init(kdq_handle* h) {
  if (!h) return KDQ_ERR_ARG;
  KDQ_CUDA(h, cudaSetDevice(h->device));
  const size_t fs = (size_t)h->Ns * h->ns;
  const bool dfl = h->precision == KDQ_PREC_MIXED;
  k_seed_chains<<<h->nchains, 256, 0, h->stream>>>(h->BRs.p, h->BLs.p, dfl ? h->Pts.p : h->Pt.p,
                                                   dfl ? h->PtHs.p : h->PtH.p, fs, h->P.sz_chainB, h->NN,
                                                   h->esz, h->P.lw);
  KDQ_CUDA(h, cudaGetLastError());
  k_reset_ctl<<<(h->nchains + 127) / 128, 128, 0, h->stream>>>(h->ctl.as<ChainCtl>(), h->nchains, 1);
  KDQ_CUDA(h, cudaGetLastError());
  h->obs_rows = 0;
  // left chain BLs[NN-1..1] and G at tau = 0  (src/tU/phy_update.jl:39-50)
  for (int k = h->NN - 1; k >= 1; --k) KDQ_CUDA(h, launch(h, KDQ_MODE_INIT, k));
  h->initialised = true;
  return KDQ_OK;
}

}  // extern "C"

namespace {

// Everything a sweep call does before its launches: argument and tape
// checks, per-call counters, the drift log and the observable rows.
int sweep_prepare(kdq_handle* h, int32_t sweeps, int32_t record) {
  if (sweeps < 0) return fail(h, KDQ_ERR_ARG, "sweeps must be >= 0");
  if (record < 0 || record > 2) return fail(h, KDQ_ERR_ARG, "record must be 0, 1 or 2");
  if (!h->initialised) return fail(h, KDQ_ERR_STATE, "kdq_init must precede kdq_sweep");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  if (h->use_tape) {
    // host-side check of the tape length against what the sweeps consume
    std::vector<ChainCtl> ctl(h->nchains);
    KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
    KDQ_CUDA(h, cudaMemcpy(ctl.data(), h->ctl.p, ctl.size() * sizeof(ChainCtl), cudaMemcpyDeviceToHost));
    const size_t need = (size_t)sweeps * 2 * h->Nt * h->n_field;
    if ((size_t)ctl[0].tape_pos + need > h->tape_len)
      return fail(h, KDQ_ERR_STATE, "proposal tape too short for the requested sweeps");
  }
  k_reset_ctl<<<(h->nchains + 127) / 128, 128, 0, h->stream>>>(h->ctl.as<ChainCtl>(), h->nchains, 0);
  KDQ_CUDA(h, cudaGetLastError());
  // drift log for this call
  const int dneed = sweeps * 2 * (h->NN - 1);
  if (dneed > h->drift_cap) {   // capacity per chain only grows, so graphs stay valid
    KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
    KDQ_CUDA(h, h->drift.alloc((size_t)dneed * h->nchains * sizeof(double)));
    h->drift_cap = dneed;
  }
  h->drift_rows = dneed;
  h->P.drift = h->drift.as<double>();
  h->P.drift_cap = h->drift_cap;
  // observables: rows for every sweep recorded since kdq_init (chain-major,
  // obs_cap rows per chain); grown by copying the old rows over
  if (record) {
    const int need_rows = h->obs_rows + sweeps;
    if (need_rows > h->obs_capacity) {
      const int cap = std::max(need_rows, 2 * h->obs_capacity);
      DevBuf nb;
      KDQ_CUDA(h, nb.alloc((size_t)cap * h->nchains * h->n_obs * sizeof(double)));
      KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
      if (h->obs_rows > 0)
        KDQ_CUDA(h, cudaMemcpy2D(nb.p, (size_t)cap * h->n_obs * sizeof(double), h->obs.p,
                                 (size_t)h->obs_capacity * h->n_obs * sizeof(double),
                                 (size_t)h->obs_rows * h->n_obs * sizeof(double), h->nchains,
                                 cudaMemcpyDeviceToDevice));
      std::swap(h->obs.p, nb.p);
      std::swap(h->obs.bytes, nb.bytes);
      h->obs_capacity = cap;
    }
    h->P.obs = h->obs.as<double>();
    h->P.obs_cap = h->obs_capacity;
  }
  if (record == 2 && !h->Lm.p) {
    const size_t NNe = (size_t)h->Ns * h->Ns, C = h->nchains;
    const int fmax = h->Nt / 2 + 1;
    const size_t stride = (((size_t)fmax * (sizeof(int) + h->n_field)) + 255) & ~(size_t)255;
    KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
    KDQ_CUDA(h, h->Lm.alloc(C * NNe * h->esz_w));
    KDQ_CUDA(h, h->Rm.alloc(C * NNe * h->esz_w));
    KDQ_CUDA(h, h->mstack.alloc(C * stride));
    h->P.Lm = h->Lm.p;
    h->P.Rm = h->Rm.p;
    h->P.mstack = h->mstack.as<uint8_t>();
    h->P.mstack_stride = stride;
    h->P.mstack_max = fmax;
  }
  h->P.record = record;
  return KDQ_OK;
}

// One sweep on the handle's stream: 2 (NN-1) block launches, or (per-sweep
// shape) a single launch in which every CTA runs its chain's blocks
// (chains are independent, so no CTA waits for another between blocks).
cudaError_t sweep_launches(kdq_handle* h) {
  if (h->sweep_launch) return launch(h, KDQ_MODE_SWEEP, 0);
  cudaError_t ce = cudaSuccess;
  for (int k = 1; k <= h->NN - 1 && ce == cudaSuccess; ++k) ce = launch(h, KDQ_MODE_FWD, k);
  for (int k = h->NN - 1; k >= 1 && ce == cudaSuccess; --k) ce = launch(h, KDQ_MODE_BWD, k);
  return ce;
}

}  // namespace

extern "C" {

int kdq_sweep(kdq_handle* h, int32_t sweeps, int32_t record) {
  if (!h) return KDQ_ERR_ARG;
  int rc = sweep_prepare(h, sweeps, record);
  if (rc) return rc;
  auto t0 = std::chrono::steady_clock::now();
  if (h->use_graphs && sweeps > 0) {
    if (!h->graph || std::memcmp(&h->graph_P, &h->P, sizeof(SweepParams)) != 0) {
      if (h->graph) {
        KDQ_CUDA(h, cudaGraphExecDestroy(h->graph));
        h->graph = nullptr;
      }
      cudaGraph_t g = nullptr;
      KDQ_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      cudaError_t ce = sweep_launches(h);
      cudaError_t ee = cudaStreamEndCapture(h->stream, &g);
      if (ce != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return cuda_fail(h, ce, "sweep capture");
      }
      KDQ_CUDA(h, ee);
      cudaError_t ie = cudaGraphInstantiate(&h->graph, g, 0);
      cudaGraphDestroy(g);
      KDQ_CUDA(h, ie);
      h->graph_P = h->P;
    }
    for (int w = 0; w < sweeps; ++w) KDQ_CUDA(h, cudaGraphLaunch(h->graph, h->stream));
  } else {
    for (int w = 0; w < sweeps; ++w) KDQ_CUDA(h, sweep_launches(h));
  }
  if (record) h->obs_rows += sweeps;
  h->last_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return KDQ_OK;
}

int kdq_synchronize(kdq_handle* h) {
  if (!h) return KDQ_ERR_ARG;
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<ChainCtl> ctl(h->nchains);
  KDQ_CUDA(h, cudaMemcpy(ctl.data(), h->ctl.p, ctl.size() * sizeof(ChainCtl), cudaMemcpyDeviceToHost));
  int flags = 0;
  for (auto& c : ctl) flags |= c.err;
  if (flags & KDQ_FLAG_TAPE) return fail(h, KDQ_ERR_STATE, "proposal tape exhausted");
  if (flags & KDQ_FLAG_NAN) return fail(h, KDQ_ERR_NUMERIC, "non-finite acceptance ratio");
  if (flags & KDQ_FLAG_SINGULAR) return fail(h, KDQ_ERR_NUMERIC, "singular BL*BR in the G recompute");
  return KDQ_OK;
}

int kdq_get_obs(kdq_handle* h, double* obs, size_t obs_len) {
  if (!h || !obs) return fail(h, KDQ_ERR_ARG, "NULL argument");
  const size_t want = (size_t)h->nchains * h->obs_rows * h->n_obs;
  if (obs_len < want) return fail(h, KDQ_ERR_ARG, "obs buffer too small: need " + std::to_string(want));
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  if (want == 0) return KDQ_OK;
  KDQ_CUDA(h, cudaMemcpy2D(obs, (size_t)h->obs_rows * h->n_obs * sizeof(double), h->obs.p,
                           (size_t)h->obs_capacity * h->n_obs * sizeof(double),
                           (size_t)h->obs_rows * h->n_obs * sizeof(double), h->nchains,
                           cudaMemcpyDeviceToHost));
  return KDQ_OK;
}

int kdq_phy_update(kdq_handle* h, int32_t sweeps, int32_t record, double* obs, size_t obs_len) {
  if (!h) return KDQ_ERR_ARG;
  if (record && (!obs || obs_len < (size_t)h->nchains * sweeps * h->n_obs))
    return fail(h, KDQ_ERR_ARG, "obs buffer too small");
  auto t0 = std::chrono::steady_clock::now();
  int rc = kdq_init(h);
  if (rc) return rc;
  rc = kdq_sweep(h, sweeps, record);
  if (rc) return rc;
  rc = kdq_synchronize(h);
  if (rc) return rc;
  if (record) {
    rc = kdq_get_obs(h, obs, obs_len);
    if (rc) return rc;
  }
  h->last_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return KDQ_OK;
}

int kdq_get_green(kdq_handle* h, int32_t chain, double* G, size_t len) {
  if (!h || !G) return fail(h, KDQ_ERR_ARG, "NULL argument");
  if (chain < 0 || chain >= h->nchains) return fail(h, KDQ_ERR_ARG, "chain out of range");
  const size_t n = (size_t)h->Ns * h->Ns * (h->gc ? 2 : 1);
  if (len != n) return fail(h, KDQ_ERR_ARG, "G buffer must hold " + std::to_string(n) + " doubles");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  const uint8_t* src = static_cast<uint8_t*>(h->G.p) + (size_t)chain * h->Ns * h->Ns * h->esz_w;
  if (h->esz_w == h->esz) {
    KDQ_CUDA(h, cudaMemcpy(G, src, n * sizeof(double), cudaMemcpyDeviceToHost));
  } else {   // working precision is FP32
    std::vector<float> f(n);
    KDQ_CUDA(h, cudaMemcpy(f.data(), src, n * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t i = 0; i < n; ++i) G[i] = f[i];
  }
  return KDQ_OK;
}

int kdq_get_drift(kdq_handle* h, double* drift, size_t len) {
  if (!h || !drift) return fail(h, KDQ_ERR_ARG, "NULL argument");
  const size_t n = (size_t)h->drift_rows * h->nchains;
  if (len != n) return fail(h, KDQ_ERR_ARG, "drift buffer must hold " + std::to_string(n) + " doubles");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  if (n)
    KDQ_CUDA(h, cudaMemcpy2D(drift, (size_t)h->drift_rows * sizeof(double), h->drift.p,
                             (size_t)h->drift_cap * sizeof(double), (size_t)h->drift_rows * sizeof(double),
                             h->nchains, cudaMemcpyDeviceToHost));
  return KDQ_OK;
}

int kdq_set_precision(kdq_handle* h, int32_t mode) {
  if (!h) return KDQ_ERR_ARG;
  if (mode != KDQ_PREC_FP64 && mode != KDQ_PREC_MIXED) return fail(h, KDQ_ERR_ARG, "unknown precision mode");
  if (mode == KDQ_PREC_MIXED && !h->gc)
    return fail(h, KDQ_ERR_ARG,
                "mixed precision needs the unitary HS factors of the complex sweeps (t-U, t-UV with U > 0); "
                "the real HS factors exp(+-alpha eta) of t-V and real t-UV amplify FP32 rounding in the "
                "wraps by the block's condition number (FP64 drift at n_wrap = 10 is already ~1e-6)");
  if (mode == h->precision) return KDQ_OK;
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  if (h->P.slmc_moves > 0)
    KDQ_CUDA(h, mode == KDQ_PREC_MIXED ? kdq::prepare_tu_mixed(h->dyn) : kdq::prepare_tu(h->dyn));
  const size_t C = h->nchains, NNe = (size_t)h->Ns * h->Ns, Nn = (size_t)h->Ns * h->ns;
  h->esz_w = mode == KDQ_PREC_MIXED ? h->esz / 2 : h->esz;
  KDQ_CUDA(h, h->G.alloc(C * NNe * h->esz_w));
  KDQ_CUDA(h, cudaMemset(h->G.p, 0, C * NNe * h->esz_w));
  KDQ_CUDA(h, h->W1.alloc(C * NNe * h->esz_w));
  KDQ_CUDA(h, h->W2.alloc(C * NNe * h->esz_w));
  h->Lm.alloc(0);
  h->Rm.alloc(0);
  h->mstack.alloc(0);
  h->P.Lm = h->P.Rm = nullptr;
  h->P.mstack = nullptr;
  SweepParams& P = h->P;
  P.G = h->G.p;
  P.W1 = h->W1.p;
  P.W2 = h->W2.p;
  if (mode == KDQ_PREC_MIXED) {
    KDQ_CUDA(h, h->Yw.alloc(C * Nn * h->esz_w));
    KDQ_CUDA(h, h->Y2w.alloc(C * Nn * h->esz_w));
    KDQ_CUDA(h, h->Gd.alloc(C * NNe * h->esz));
    const size_t kn = NNe * (h->kc ? 2 : 1);   // doubles per kinetic matrix
    DevBuf* dst[4] = {&h->eKw, &h->eKinvw, &h->HalfeKw, &h->HalfeKinvw};
    DevBuf* src[4] = {&h->eK, &h->eKinv, &h->HalfeK, &h->HalfeKinv};
    for (int q = 0; q < 4; ++q) {
      KDQ_CUDA(h, dst[q]->alloc(kn * sizeof(float)));
      k_to_float<<<64, 256, 0, h->stream>>>(src[q]->as<double>(), dst[q]->as<float>(), kn);
      KDQ_CUDA(h, cudaGetLastError());
    }
    if (!h->kc) {   // real kinetic matrices: pre-split operands of the tensor-core products
      const size_t words = kdq::kin_frag_words(h->Ns);
      KDQ_CUDA(h, h->kinfrag.alloc(8 * words * sizeof(uint4)));
      uint4* base = h->kinfrag.as<uint4>();
      for (int q = 0; q < 4; ++q) {
        k_kin_frag<<<64, 256, 0, h->stream>>>(dst[q]->as<float>(), h->Ns, base + (size_t)(2 * q) * words,
                                              base + (size_t)(2 * q + 1) * words);
        KDQ_CUDA(h, cudaGetLastError());
      }
      P.kin_frag = base;
      P.kin_frag_words = words;
    } else {
      h->kinfrag.alloc(0);
      P.kin_frag = nullptr;
      P.kin_frag_words = 0;
    }
    const size_t pn = Nn * (h->gc ? 2 : 1);   // doubles per trial-state matrix
    KDQ_CUDA(h, h->Pts.alloc(pn * 2 * sizeof(float)));
    KDQ_CUDA(h, h->PtHs.alloc(pn * 2 * sizeof(float)));
    k_to_dfl<<<64, 256, 0, h->stream>>>(h->Pt.as<double>(), h->Pts.as<float>(), pn);
    KDQ_CUDA(h, cudaGetLastError());
    k_to_dfl<<<64, 256, 0, h->stream>>>(h->PtH.as<double>(), h->PtHs.as<float>(), pn);
    KDQ_CUDA(h, cudaGetLastError());
    P.Yw = h->Yw.p;
    P.Y2w = h->Y2w.p;
    P.Gd = h->Gd.p;
    P.eK = h->eKw.p;
    P.eKinv = h->eKinvw.p;
    P.HalfeK = h->HalfeKw.p;
    P.HalfeKinv = h->HalfeKinvw.p;
  } else {
    h->Yw.alloc(0);
    h->Y2w.alloc(0);
    h->Gd.alloc(0);
    h->Pts.alloc(0);
    h->PtHs.alloc(0);
    h->kinfrag.alloc(0);
    P.kin_frag = nullptr;
    P.kin_frag_words = 0;
    P.Yw = h->Y.p;
    P.Y2w = h->Y2.p;
    P.Gd = h->W1.p;
    P.eK = h->eK.p;
    P.eKinv = h->eKinv.p;
    P.HalfeK = h->HalfeK.p;
    P.HalfeKinv = h->HalfeKinv.p;
  }
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  h->precision = mode;
  h->initialised = false;
  return KDQ_OK;
}

int kdq_enable_phase_timing(kdq_handle* h, int32_t enable) {
  if (!h) return KDQ_ERR_ARG;
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  if (enable) {
    KDQ_CUDA(h, h->phase.alloc((size_t)h->nchains * 8 * sizeof(unsigned long long)));
    KDQ_CUDA(h, cudaMemset(h->phase.p, 0, h->phase.bytes));
    h->P.phase = h->phase.as<unsigned long long>();
  } else {
    h->phase.alloc(0);
    h->P.phase = nullptr;
  }
  return KDQ_OK;
}

int kdq_get_phase_cycles(kdq_handle* h, double* cycles) {
  if (!h || !cycles) return fail(h, KDQ_ERR_ARG, "NULL argument");
  if (!h->P.phase) return fail(h, KDQ_ERR_STATE, "phase timing is not enabled");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<unsigned long long> v((size_t)h->nchains * 8);
  KDQ_CUDA(h, cudaMemcpy(v.data(), h->phase.p, v.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  for (int q = 0; q < 8; ++q) cycles[q] = 0.0;
  for (int c = 0; c < h->nchains; ++c)
    for (int q = 0; q < 8; ++q) cycles[q] += (double)v[(size_t)c * 8 + q];
  return KDQ_OK;
}

int kdq_set_graphs(kdq_handle* h, int32_t enable) {
  if (!h) return KDQ_ERR_ARG;
  h->use_graphs = enable != 0;
  return KDQ_OK;
}

int kdq_set_sweep_launch(kdq_handle* h, int32_t per_sweep) {
  if (!h) return KDQ_ERR_ARG;
  if (h->sweep_launch != (per_sweep != 0) && h->graph) {   // the captured sweep has the other shape
    KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
    KDQ_CUDA(h, cudaGraphExecDestroy(h->graph));
    h->graph = nullptr;
  }
  h->sweep_launch = per_sweep != 0;
  return KDQ_OK;
}

int kdq_get_stats(kdq_handle* h, kdq_stats* st) {
  if (!h || !st) return fail(h, KDQ_ERR_ARG, "NULL argument");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<ChainCtl> ctl(h->nchains);
  KDQ_CUDA(h, cudaMemcpy(ctl.data(), h->ctl.p, ctl.size() * sizeof(ChainCtl), cudaMemcpyDeviceToHost));
  std::memset(st, 0, sizeof(*st));
  for (auto& c : ctl) {
    st->proposals += c.n_prop;
    st->accepted += c.n_acc;
    st->recomputes += c.n_recompute;
    if (!(c.max_drift <= st->max_drift)) st->max_drift = c.max_drift;
  }
  st->seconds = h->last_seconds;
  return KDQ_OK;
}

int kdq_get_log_det(kdq_handle* h, double* logdet, double* phase, size_t len) {
  if (!h || !logdet || !phase) return fail(h, KDQ_ERR_ARG, "NULL argument");
  if (len != (size_t)h->nchains) return fail(h, KDQ_ERR_ARG, "len must equal the number of chains");
  if (!h->initialised) return fail(h, KDQ_ERR_STATE, "kdq_init must precede kdq_get_log_det");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<ChainCtl> ctl(h->nchains);
  KDQ_CUDA(h, cudaMemcpy(ctl.data(), h->ctl.p, ctl.size() * sizeof(ChainCtl), cudaMemcpyDeviceToHost));
  for (size_t c = 0; c < ctl.size(); ++c) {
    logdet[c] = ctl[c].logdet;
    phase[2 * c] = ctl[c].det_re;
    phase[2 * c + 1] = ctl[c].det_im;
  }
  return KDQ_OK;
}

namespace {
uint16_t to_bf16_bits(float f) {   // round to nearest even (finite values)
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
}  // namespace

int kdq_slmc_enable(kdq_handle* h, const float* params, int32_t moves_per_slice, int32_t cluster_len,
                    int32_t eff_steps) {
  if (!h) return KDQ_ERR_ARG;
  if (moves_per_slice < 0) return fail(h, KDQ_ERR_ARG, "moves_per_slice must be >= 0");
  if (moves_per_slice == 0) {
    KDQ_CUDA(h, cudaSetDevice(h->device));
    KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
    h->P.slmc_moves = 0;
    h->dyn = h->dyn_base;
    return KDQ_OK;
  }
  if (h->kind != KDQ_TU) return fail(h, KDQ_ERR_ARG, "self-learning cluster moves are implemented for t-U only");
  if (!params) return fail(h, KDQ_ERR_ARG, "NULL params");
  const int lmax = std::min(32, std::min(h->ns, h->Ns - 8));
  if (cluster_len < 1 || cluster_len > lmax)
    return fail(h, KDQ_ERR_ARG, "cluster_len must be in [1, min(32, Ns/2, Ns-8)] = [1, " + std::to_string(lmax) + "]");
  if (h->Nt < 9) return fail(h, KDQ_ERR_ARG, "cluster moves need Nt >= 9");
  if (eff_steps < 1 || eff_steps > (1 << 20)) return fail(h, KDQ_ERR_ARG, "eff_steps must be in [1, 2^20]");
  for (int i = 0; i < KDQ_CNN_PARAMS; ++i)
    if (!std::isfinite(params[i])) return fail(h, KDQ_ERR_ARG, "non-finite effective-model parameter");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<uint16_t> b(KDQ_CNN_PARAMS);
  for (int i = 0; i < KDQ_CNN_PARAMS; ++i) b[i] = to_bf16_bits(params[i]);
  if (!h->slmc_prm.p) KDQ_CUDA(h, h->slmc_prm.alloc(b.size() * sizeof(uint16_t)));
  KDQ_CUDA(h, cudaMemcpy(h->slmc_prm.p, b.data(), b.size() * sizeof(uint16_t), cudaMemcpyHostToDevice));
  const size_t off = (h->dyn_base + 15) & ~(size_t)15;
  const size_t dyn = off + kdq::slmc_smem_bytes(cluster_len);
  KDQ_CUDA(h, h->precision == KDQ_PREC_MIXED ? kdq::prepare_tu_mixed(dyn) : kdq::prepare_tu(dyn));
  h->P.slmc_moves = moves_per_slice;
  h->P.slmc_len = cluster_len;
  h->P.slmc_steps = eff_steps;
  h->P.slmc_off = off;
  h->P.slmc_prm = h->slmc_prm.p;
  h->dyn = dyn;
  return KDQ_OK;
}

namespace {
// shared set-up of the coupled SCEE sweep (dop = 0: replica pairs) and the
// disorder-operator sweep (dop = 1: single chains)
int scee_setup(kdq_handle* h, const int32_t* indexA, int32_t nA, const int32_t* indexB, int32_t nB, double lambda,
               int32_t n_lambda, int dop, double alpha) {
  if (!h) return KDQ_ERR_ARG;
  if (dop && h->kind != KDQ_TU) return fail(h, KDQ_ERR_ARG, "the disorder-operator sweep is implemented for t-U");
  if (!dop && h->nchains % 2) return fail(h, KDQ_ERR_ARG, "the SCEE sweep needs an even number of chains (replica pairs)");
  if (!std::isfinite(alpha)) return fail(h, KDQ_ERR_ARG, "alpha must be finite");
  if (h->precision != KDQ_PREC_FP64) return fail(h, KDQ_ERR_ARG, "the SCEE sweep runs in FP64 only");
  if (!indexA || !indexB) return fail(h, KDQ_ERR_ARG, "NULL region");
  const int nmax_ok = std::min(h->ns, 96);
  if (nA < 1 || nB < 1 || nA > nmax_ok || nB > nmax_ok)
    return fail(h, KDQ_ERR_ARG, "region sizes must be in [1, min(Ns/2, 96)] = [1, " + std::to_string(nmax_ok) + "]");
  std::vector<int32_t> idx;
  for (int i = 0; i < nA; ++i) idx.push_back(indexA[i] - 1);
  for (int i = 0; i < nB; ++i) idx.push_back(indexB[i] - 1);
  for (int v : idx)
    if (v < 0 || v >= h->Ns) return fail(h, KDQ_ERR_ARG, "region index out of range (1-based)");
  if (!(lambda >= 0.0 && lambda <= 1.0)) return fail(h, KDQ_ERR_ARG, "lambda must be in [0, 1]");
  if (n_lambda < 1) return fail(h, KDQ_ERR_ARG, "n_lambda must be >= 1");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  const size_t C = h->nchains, NN2 = (size_t)h->Ns * h->Ns, e = h->esz, pairs = dop ? C : C / 2;
  const int nmax = std::max(nA, nB);
  if (!h->scee) {
    KDQ_CUDA(h, h->scee_G0.alloc(C * NN2 * e));
    KDQ_CUDA(h, h->scee_Gt0.alloc(C * NN2 * e));
    KDQ_CUDA(h, h->scee_G0t.alloc(C * NN2 * e));
    KDQ_CUDA(h, h->scee_BMs.alloc(C * (h->NN - 1) * NN2 * e));
    KDQ_CUDA(h, h->scee_BMi.alloc(C * (h->NN - 1) * NN2 * e));
  }
  KDQ_CUDA(h, h->scee_det.alloc(pairs * 4 * sizeof(double)));
  KDQ_CUDA(h, h->scee_inv.alloc(pairs * 2 * (size_t)nmax * nmax * e));
  KDQ_CUDA(h, upload(h->scee_idx, idx));
  SweepParams& P = h->P;
  P.scee_G0 = h->scee_G0.p;
  P.scee_Gt0 = h->scee_Gt0.p;
  P.scee_G0t = h->scee_G0t.p;
  P.scee_BMs = h->scee_BMs.p;
  P.scee_BMi = h->scee_BMi.p;
  P.scee_inv = h->scee_inv.p;
  P.scee_idxA = h->scee_idx.as<int32_t>();
  P.scee_idxB = h->scee_idx.as<int32_t>() + nA;
  P.scee_nA = nA;
  P.scee_nB = nB;
  P.scee_nmax = nmax;
  P.scee_nlam = n_lambda;
  P.scee_lam = lambda;
  P.scee_det = h->scee_det.as<double>();
  P.scee_dop = dop;
  P.scee_alpha = alpha;
  h->scee_lam = lambda;
  h->scee = true;
  return KDQ_OK;
}

int scee_run(kdq_handle* h, int32_t sweeps, double* O, size_t len, int dop) {
  if (!h) return KDQ_ERR_ARG;
  if (!h->scee || h->P.scee_dop != dop)
    return fail(h, KDQ_ERR_STATE, dop ? "kdq_dop_enable must precede kdq_dop_run" : "kdq_scee_enable must precede kdq_scee_run");
  if (sweeps < 0) return fail(h, KDQ_ERR_ARG, "sweeps must be >= 0");
  const size_t pairs = dop ? h->nchains : h->nchains / 2;
  if (!O || len != pairs * (size_t)(sweeps + 1))
    return fail(h, KDQ_ERR_ARG, dop ? "O must hold n_chains * (sweeps + 1) doubles" : "O must hold n_pairs * (sweeps + 1) doubles");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  if (h->use_tape) {
    std::vector<ChainCtl> ctl(h->nchains);
    KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
    KDQ_CUDA(h, cudaMemcpy(ctl.data(), h->ctl.p, ctl.size() * sizeof(ChainCtl), cudaMemcpyDeviceToHost));
    if ((size_t)ctl[0].tape_pos + (size_t)sweeps * 2 * h->Nt * h->Ns > h->tape_len)
      return fail(h, KDQ_ERR_STATE, "proposal tape too short for the requested sweeps");
  }
  const size_t fs = (size_t)h->Ns * h->ns;
  k_seed_chains<<<h->nchains, 256, 0, h->stream>>>(h->BRs.p, h->BLs.p, h->Pt.p, h->PtH.p, fs, h->P.sz_chainB,
                                                   h->NN, h->esz, h->P.lw);
  KDQ_CUDA(h, cudaGetLastError());
  k_reset_ctl<<<(h->nchains + 127) / 128, 128, 0, h->stream>>>(h->ctl.as<ChainCtl>(), h->nchains, 1);
  KDQ_CUDA(h, cudaGetLastError());
  KDQ_CUDA(h, h->scee_O.alloc(pairs * (size_t)std::max(sweeps, 1) * sizeof(double)));
  KDQ_CUDA(h, cudaMemsetAsync(h->scee_det.p, 0, pairs * 4 * sizeof(double), h->stream));
  SweepParams P = h->P;
  P.scee_O = h->scee_O.as<double>();
  P.scee_O_cap = std::max(sweeps, 1);
  P.record = 0;
  const bool kc = h->kc;
  auto t0 = std::chrono::steady_clock::now();
  KDQ_CUDA(h, kdq::launch_scee(P, KDQ_MODE_INIT, 0, h->maxrm, kc, h->gc, (int)pairs, h->stream));
  for (int w = 0; w < sweeps; ++w) {
    for (int k = 1; k <= h->NN - 1; ++k) KDQ_CUDA(h, kdq::launch_scee(P, KDQ_MODE_FWD, k, h->maxrm, kc, h->gc, (int)pairs, h->stream));
    for (int k = h->NN - 1; k >= 1; --k) KDQ_CUDA(h, kdq::launch_scee(P, KDQ_MODE_BWD, k, h->maxrm, kc, h->gc, (int)pairs, h->stream));
  }
  if (int rc = kdq_synchronize(h)) return rc;
  h->last_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::vector<double> rows(pairs * (size_t)std::max(sweeps, 1));
  if (sweeps > 0)
    KDQ_CUDA(h, cudaMemcpy(rows.data(), h->scee_O.p, rows.size() * sizeof(double), cudaMemcpyDeviceToHost));
  for (size_t p = 0; p < pairs; ++p) {
    O[p * (sweeps + 1)] = h->scee_lam;
    for (int w = 0; w < sweeps; ++w) O[p * (sweeps + 1) + 1 + w] = rows[p * std::max(sweeps, 1) + w];
  }
  h->initialised = false;   // G and the chains now hold the SCEE state
  return KDQ_OK;
}
}  // namespace

int kdq_scee_enable(kdq_handle* h, const int32_t* indexA, int32_t nA, const int32_t* indexB, int32_t nB,
                    double lambda, int32_t n_lambda) {
  return scee_setup(h, indexA, nA, indexB, nB, lambda, n_lambda, 0, 0.0);
}

int kdq_scee_run(kdq_handle* h, int32_t sweeps, double* O, size_t len) { return scee_run(h, sweeps, O, len, 0); }

int kdq_dop_enable(kdq_handle* h, double alpha, const int32_t* indexA, int32_t nA, const int32_t* indexB,
                   int32_t nB, double lambda, int32_t n_lambda) {
  return scee_setup(h, indexA, nA, indexB, nB, lambda, n_lambda, 1, alpha);
}

int kdq_dop_run(kdq_handle* h, int32_t sweeps, double* O, size_t len) { return scee_run(h, sweeps, O, len, 1); }

int kdq_scee_get_green(kdq_handle* h, int32_t chain, int32_t which, double* G, size_t len) {
  if (!h || !G) return fail(h, KDQ_ERR_ARG, "NULL argument");
  if (!h->scee) return fail(h, KDQ_ERR_STATE, "kdq_scee_enable must precede kdq_scee_get_green");
  if (chain < 0 || chain >= h->nchains || which < 0 || which > 3) return fail(h, KDQ_ERR_ARG, "chain or which out of range");
  const size_t NN2 = (size_t)h->Ns * h->Ns;
  if (len != NN2 * (h->esz / 8)) return fail(h, KDQ_ERR_ARG, "G must hold Ns^2 values (2 doubles each if complex)");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  const DevBuf* src[4] = {&h->G, &h->scee_G0, &h->scee_Gt0, &h->scee_G0t};
  KDQ_CUDA(h, cudaMemcpy(G, static_cast<const uint8_t*>(src[which]->p) + (size_t)chain * NN2 * h->esz,
                         NN2 * h->esz, cudaMemcpyDeviceToHost));
  return KDQ_OK;
}

int kdq_set_measure_full(kdq_handle* h, int32_t enable) {
  if (!h) return KDQ_ERR_ARG;
  if (h->kind == KDQ_TV || (h->kind == KDQ_TUV && !h->gc))
    return fail(h, KDQ_ERR_ARG, "the full structure factors are measured for t-U and complex t-UV only");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  h->P.meas_full = enable ? 1 : 0;
  h->n_obs = (h->kind == KDQ_TU ? 6 : 7) + (enable ? 4 : 0);
  h->P.n_obs = h->n_obs;
  h->obs_rows = 0;        // rows of the other width are dropped
  h->obs_capacity = 0;
  return KDQ_OK;
}

int kdq_get_slmc_stats(kdq_handle* h, int64_t* counts) {
  if (!h || !counts) return fail(h, KDQ_ERR_ARG, "NULL argument");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  std::vector<ChainCtl> ctl(h->nchains);
  KDQ_CUDA(h, cudaMemcpy(ctl.data(), h->ctl.p, ctl.size() * sizeof(ChainCtl), cudaMemcpyDeviceToHost));
  counts[0] = counts[1] = counts[2] = 0;
  for (auto& c : ctl) {
    counts[0] += c.slmc_prop;
    counts[1] += c.slmc_acc;
    counts[2] += c.slmc_noop;
  }
  return KDQ_OK;
}

// ------------------------------------------------------------ Grover det
namespace {
int check_region(const int32_t* index, int32_t nA, int32_t Ns, std::string& why) {
  if (!index || nA < 1 || nA > Ns) { why = "region size must be in [1, Ns]"; return 1; }
  for (int i = 0; i < nA; ++i)
    if (index[i] < 1 || index[i] > Ns) { why = "region index out of range (1-based)"; return 1; }
  return 0;
}
}  // namespace

int kdq_grover_det(const double* G, int32_t Ns, int32_t g_complex, int32_t npairs, const int32_t* index,
                   int32_t nA, double* det, int32_t device) {
  auto set_err = [](int code, const std::string& msg) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_err = msg;
    return code;
  };
  std::string why;
  if (!G || !det) return set_err(KDQ_ERR_ARG, "NULL argument");
  if (Ns < 2 || npairs < 0) return set_err(KDQ_ERR_ARG, "bad sizes");
  if (check_region(index, nA, Ns, why)) return set_err(KDQ_ERR_ARG, why);
  if (npairs == 0) return KDQ_OK;
  if (cudaSetDevice(device) != cudaSuccess) return set_err(KDQ_ERR_NOGPU, "cannot select device");
  const size_t esz = g_complex ? 16 : 8;
  const size_t gbytes = (size_t)2 * npairs * Ns * Ns * esz;
  std::vector<int> idx0(nA);
  for (int i = 0; i < nA; ++i) idx0[i] = index[i] - 1;
  DevBuf dG, dScr, dPiv, dIdx, dDet;
  cudaError_t e;
  if ((e = dG.alloc(gbytes)) || (e = dScr.alloc(kdq::grover_scratch_bytes(nA, npairs, g_complex))) ||
      (e = dPiv.alloc((size_t)npairs * nA * sizeof(int))) || (e = dIdx.alloc((size_t)nA * sizeof(int))) ||
      (e = dDet.alloc((size_t)2 * npairs * sizeof(double))))
    return set_err(KDQ_ERR_CUDA, cudaGetErrorString(e));
  if ((e = cudaMemcpy(dG.p, G, gbytes, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(dIdx.p, idx0.data(), (size_t)nA * sizeof(int), cudaMemcpyHostToDevice)) ||
      (e = kdq::launch_grover(dG.p, Ns, g_complex != 0, dIdx.as<int>(), nA, npairs, dScr.p, dPiv.as<int>(),
                              dDet.as<double>(), nullptr)) ||
      (e = cudaMemcpy(det, dDet.p, (size_t)2 * npairs * sizeof(double), cudaMemcpyDeviceToHost)))
    return set_err(KDQ_ERR_CUDA, cudaGetErrorString(e));
  return KDQ_OK;
}

int kdq_keep_middle_green(kdq_handle* h, int32_t enable) {
  if (!h) return KDQ_ERR_ARG;
  KDQ_CUDA(h, cudaSetDevice(h->device));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  if (enable) {
    const size_t b = (size_t)h->nchains * h->Ns * h->Ns * h->esz;
    if (h->gmid.bytes != b) KDQ_CUDA(h, h->gmid.alloc(b));
    KDQ_CUDA(h, cudaMemset(h->gmid.p, 0, b));
    h->P.gmid = h->gmid.p;
  } else {
    h->gmid.alloc(0);
    h->P.gmid = nullptr;
  }
  return KDQ_OK;
}

int kdq_grover_det_middle(kdq_handle* h, const int32_t* index, int32_t nA, double* det) {
  if (!h || !det) return fail(h, KDQ_ERR_ARG, "NULL argument");
  if (!h->P.gmid) return fail(h, KDQ_ERR_STATE, "kdq_keep_middle_green is not enabled");
  std::string why;
  if (check_region(index, nA, h->Ns, why)) return fail(h, KDQ_ERR_ARG, why);
  const int npairs = h->nchains / 2;
  if (npairs == 0) return fail(h, KDQ_ERR_ARG, "need at least two chains");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  const size_t sb = kdq::grover_scratch_bytes(nA, npairs, h->gc);
  if (h->gr_scratch.bytes < sb) KDQ_CUDA(h, h->gr_scratch.alloc(sb));
  if (h->gr_piv.bytes < (size_t)npairs * nA * sizeof(int)) KDQ_CUDA(h, h->gr_piv.alloc((size_t)npairs * nA * sizeof(int)));
  if (h->gr_index.bytes < (size_t)nA * sizeof(int)) KDQ_CUDA(h, h->gr_index.alloc((size_t)nA * sizeof(int)));
  if (h->gr_det.bytes < (size_t)2 * npairs * sizeof(double)) KDQ_CUDA(h, h->gr_det.alloc((size_t)2 * npairs * sizeof(double)));
  std::vector<int> idx0(nA);
  for (int i = 0; i < nA; ++i) idx0[i] = index[i] - 1;
  KDQ_CUDA(h, cudaMemcpyAsync(h->gr_index.p, idx0.data(), (size_t)nA * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  KDQ_CUDA(h, kdq::launch_grover(h->gmid.p, h->Ns, h->gc, h->gr_index.as<int>(), nA, npairs, h->gr_scratch.p,
                                 h->gr_piv.as<int>(), h->gr_det.as<double>(), h->stream));
  KDQ_CUDA(h, cudaMemcpyAsync(det, h->gr_det.p, (size_t)2 * npairs * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  return KDQ_OK;
}

int kdq_grover_det_chains(kdq_handle* h, const int32_t* index, int32_t nA, double* det) {
  if (!h || !det) return fail(h, KDQ_ERR_ARG, "NULL argument");
  std::string why;
  if (check_region(index, nA, h->Ns, why)) return fail(h, KDQ_ERR_ARG, why);
  const int npairs = h->nchains / 2;
  if (npairs == 0) return fail(h, KDQ_ERR_ARG, "need at least two chains");
  KDQ_CUDA(h, cudaSetDevice(h->device));
  const size_t sb = kdq::grover_scratch_bytes(nA, npairs, h->gc);
  if (h->gr_scratch.bytes < sb) KDQ_CUDA(h, h->gr_scratch.alloc(sb));
  if (h->gr_piv.bytes < (size_t)npairs * nA * sizeof(int)) KDQ_CUDA(h, h->gr_piv.alloc((size_t)npairs * nA * sizeof(int)));
  if (h->gr_index.bytes < (size_t)nA * sizeof(int)) KDQ_CUDA(h, h->gr_index.alloc((size_t)nA * sizeof(int)));
  if (h->gr_det.bytes < (size_t)2 * npairs * sizeof(double)) KDQ_CUDA(h, h->gr_det.alloc((size_t)2 * npairs * sizeof(double)));
  std::vector<int> idx0(nA);
  for (int i = 0; i < nA; ++i) idx0[i] = index[i] - 1;
  KDQ_CUDA(h, cudaMemcpyAsync(h->gr_index.p, idx0.data(), (size_t)nA * sizeof(int), cudaMemcpyHostToDevice, h->stream));
  KDQ_CUDA(h, kdq::launch_grover(h->G.p, h->Ns, h->gc, h->gr_index.as<int>(), nA, npairs, h->gr_scratch.p,
                                 h->gr_piv.as<int>(), h->gr_det.as<double>(), h->stream));
  KDQ_CUDA(h, cudaMemcpyAsync(det, h->gr_det.p, (size_t)2 * npairs * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
  return KDQ_OK;
}

// ------------------------------------------------------------ tile classes
int kdq_set_tiles(kdq_handle* h, int32_t rows) {
  if (!h) return KDQ_ERR_ARG;
  if (rows != 1 && rows != 3 && rows != 6) return fail(h, KDQ_ERR_ARG, "tile class must be 1, 3 or 6");
  if (32 * rows < h->Ns)
    return fail(h, KDQ_ERR_ARG, "tile class " + std::to_string(rows) + " covers at most " +
                                    std::to_string(32 * rows) + " sites");
  if (rows != h->maxrm) {
    KDQ_CUDA(h, cudaSetDevice(h->device));
    KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
    h->maxrm = rows;
    if (h->graph) {   // the captured sweep launches the old instantiation
      KDQ_CUDA(h, cudaGraphExecDestroy(h->graph));
      h->graph = nullptr;
    }
  }
  return KDQ_OK;
}

int kdq_get_tiles(const kdq_handle* h) { return h ? h->maxrm : 0; }

int kdq_autotune(kdq_handle* h, int32_t* chosen, double* ms, int32_t len) {
  if (!h) return KDQ_ERR_ARG;
  static const int cand[3] = {1, 3, 6};
  const TuneKey key{h->device, h->kind, h->Ns, h->Nt, h->gc, h->kc, h->precision, h->nchains, h->P.slmc_moves};
  double t[3] = {-1.0, -1.0, -1.0};
  int best = -1;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (auto& e : g_tune)
      if (e.key == key) {
        best = e.rows;
        for (int i = 0; i < 3; ++i) t[i] = e.ms[i];
      }
  }
  KDQ_CUDA(h, cudaSetDevice(h->device));
  if (best < 0) {
    // time one sweep per valid class on the handle's own chains, then put
    // the fields and the per-chain counters (RNG position) back
    KDQ_CUDA(h, cudaStreamSynchronize(h->stream));
    const size_t fbytes = (size_t)h->nchains * h->Nt * h->n_field;
    const size_t cbytes = (size_t)h->nchains * sizeof(ChainCtl);
    DevBuf s0, c0;
    KDQ_CUDA(h, s0.alloc(fbytes));
    KDQ_CUDA(h, c0.alloc(cbytes));
    KDQ_CUDA(h, cudaMemcpyAsync(s0.p, h->s.p, fbytes, cudaMemcpyDeviceToDevice, h->stream));
    KDQ_CUDA(h, cudaMemcpyAsync(c0.p, h->ctl.p, cbytes, cudaMemcpyDeviceToDevice, h->stream));
    const int keep = h->maxrm;
    cudaEvent_t e0, e1;
    KDQ_CUDA(h, cudaEventCreate(&e0));
    KDQ_CUDA(h, cudaEventCreate(&e1));
    int rc = KDQ_OK;
    for (int i = 0; i < 3 && rc == KDQ_OK; ++i) {
      if (32 * cand[i] < h->Ns) continue;
      if ((rc = kdq_set_tiles(h, cand[i])) != KDQ_OK) break;
      if ((rc = kdq_init(h)) != KDQ_OK) break;
      if ((rc = kdq_sweep(h, 1, 0)) != KDQ_OK) break;    // captures the graph
      cudaError_t e = cudaEventRecord(e0, h->stream);
      if (e == cudaSuccess && (rc = kdq_sweep(h, 1, 0)) != KDQ_OK) break;
      if (e == cudaSuccess) e = cudaEventRecord(e1, h->stream);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float f = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&f, e0, e1);
      if (e == cudaSuccess) e = cudaMemcpyAsync(h->s.p, s0.p, fbytes, cudaMemcpyDeviceToDevice, h->stream);
      if (e == cudaSuccess) e = cudaMemcpyAsync(h->ctl.p, c0.p, cbytes, cudaMemcpyDeviceToDevice, h->stream);
      if (e != cudaSuccess) {
        rc = cuda_fail(h, e, "autotune");
        break;
      }
      if ((rc = kdq_synchronize(h)) != KDQ_OK) break;
      t[i] = f;
      if (best < 0 || f < t[best]) best = i;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != KDQ_OK) {   // put the fields and counters back, keep the message
      const std::string msg = h->err;
      cudaStreamSynchronize(h->stream);
      cudaMemcpy(h->s.p, s0.p, fbytes, cudaMemcpyDeviceToDevice);
      cudaMemcpy(h->ctl.p, c0.p, cbytes, cudaMemcpyDeviceToDevice);
      kdq_set_tiles(h, keep);
      h->initialised = false;
      h->err = msg;
      return rc;
    }
    best = cand[best];
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.push_back({key, best, {t[0], t[1], t[2]}});
  }
  int rc = kdq_set_tiles(h, best);
  if (rc) return rc;
  if (chosen) *chosen = best;
  for (int i = 0; ms && i < len && i < 3; ++i) ms[i] = t[i];
  return kdq_init(h);
}

}  // extern "C"

// ------------------------------------------------------------ groups
namespace kdq {
void set_global_error(const std::string& msg);
}

// Handles of different lattices, models or precisions swept together: one
// CUDA graph per sweep whose branches are the handles' block launches, so
// their CTAs share the GPU in one submission.
struct kdq_group {
  int device = 0;
  std::vector<kdq_handle*> hs;
  cudaStream_t stream = nullptr;
  cudaEvent_t fork = nullptr, done = nullptr;
  std::vector<cudaEvent_t> ready, joins;
  cudaGraphExec_t graph = nullptr;
  std::vector<SweepParams> graph_P;
  std::vector<int> graph_rm, graph_prec;
  std::string err;
  ~kdq_group() {
    if (graph) cudaGraphExecDestroy(graph);
    for (auto e : ready) cudaEventDestroy(e);
    for (auto e : joins) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (done) cudaEventDestroy(done);
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace {
int gfail(kdq_group* g, int code, const std::string& msg) {
  if (g) g->err = msg;
  return code;
}
#define KDQ_GCUDA(g, call)                                                          \
  do {                                                                              \
    cudaError_t _e = (call);                                                        \
    if (_e != cudaSuccess) return gfail(g, KDQ_ERR_CUDA, std::string(#call) + ": " + \
                                              cudaGetErrorString(_e));              \
  } while (0)
}  // namespace

extern "C" {

int kdq_group_create(kdq_group** out, kdq_handle* const* handles, int32_t n) {
  if (!out || !handles || n < 1) {
    kdq::set_global_error("kdq_group_create: NULL argument or empty group");
    return KDQ_ERR_ARG;
  }
  *out = nullptr;
  for (int i = 0; i < n; ++i) {
    if (!handles[i]) {
      kdq::set_global_error("kdq_group_create: NULL handle");
      return KDQ_ERR_ARG;
    }
    for (int j = 0; j < i; ++j)
      if (handles[j] == handles[i]) {
        kdq::set_global_error("kdq_group_create: a handle appears twice");
        return KDQ_ERR_ARG;
      }
    if (handles[i]->device != handles[0]->device) {
      kdq::set_global_error("kdq_group_create: handles on different devices");
      return KDQ_ERR_ARG;
    }
  }
  auto* g = new kdq_group;
  g->device = handles[0]->device;
  g->hs.assign(handles, handles + n);
  auto bad = [&](cudaError_t e) {
    kdq::set_global_error(std::string("kdq_group_create: ") + cudaGetErrorString(e));
    delete g;
    return KDQ_ERR_CUDA;
  };
  cudaError_t e = cudaSetDevice(g->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->done, cudaEventDisableTiming);
  g->ready.assign(n, nullptr);
  g->joins.assign(n, nullptr);
  for (int i = 0; i < n && e == cudaSuccess; ++i) {
    e = cudaEventCreateWithFlags(&g->ready[i], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&g->joins[i], cudaEventDisableTiming);
  }
  if (e != cudaSuccess) return bad(e);
  *out = g;
  return KDQ_OK;
}

const char* kdq_group_last_error(const kdq_group* g) { return g ? g->err.c_str() : "NULL group"; }

void kdq_group_destroy(kdq_group* g) {
  if (!g) return;
  cudaSetDevice(g->device);
  cudaStreamSynchronize(g->stream);
  delete g;
}

int kdq_group_sweep(kdq_group* g, int32_t sweeps, int32_t record) {
  if (!g) return KDQ_ERR_ARG;
  KDQ_GCUDA(g, cudaSetDevice(g->device));
  const int n = (int)g->hs.size();
  for (int i = 0; i < n; ++i) {
    kdq_handle* h = g->hs[i];
    if (!h->initialised) return gfail(g, KDQ_ERR_STATE, "handle " + std::to_string(i) + ": kdq_init must precede the group sweep");
    if (int rc = sweep_prepare(h, sweeps, record)) return gfail(g, rc, "handle " + std::to_string(i) + ": " + h->err);
    KDQ_GCUDA(g, cudaEventRecord(g->ready[i], h->stream));
    KDQ_GCUDA(g, cudaStreamWaitEvent(g->stream, g->ready[i], 0));
  }
  bool same = g->graph != nullptr;
  for (int i = 0; same && i < n; ++i)
    same = std::memcmp(&g->graph_P[i], &g->hs[i]->P, sizeof(SweepParams)) == 0 &&
           g->graph_rm[i] == g->hs[i]->maxrm && g->graph_prec[i] == g->hs[i]->precision;
  if (sweeps > 0 && !same) {
    if (g->graph) {
      KDQ_GCUDA(g, cudaGraphExecDestroy(g->graph));
      g->graph = nullptr;
    }
    cudaGraph_t gr = nullptr;
    KDQ_GCUDA(g, cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaEventRecord(g->fork, g->stream);
    for (int i = 0; i < n && ce == cudaSuccess; ++i) {
      kdq_handle* h = g->hs[i];
      ce = cudaStreamWaitEvent(h->stream, g->fork, 0);     // the branch joins the capture
      if (ce == cudaSuccess) ce = sweep_launches(h);
      if (ce == cudaSuccess) ce = cudaEventRecord(g->joins[i], h->stream);
      if (ce == cudaSuccess) ce = cudaStreamWaitEvent(g->stream, g->joins[i], 0);
    }
    cudaError_t ee = cudaStreamEndCapture(g->stream, &gr);
    if (ce != cudaSuccess || ee != cudaSuccess) {
      if (gr) cudaGraphDestroy(gr);
      return gfail(g, KDQ_ERR_CUDA, std::string("group sweep capture: ") +
                                        cudaGetErrorString(ce != cudaSuccess ? ce : ee));
    }
    cudaError_t ie = cudaGraphInstantiate(&g->graph, gr, 0);
    cudaGraphDestroy(gr);
    KDQ_GCUDA(g, ie);
    g->graph_P.resize(n);
    g->graph_rm.resize(n);
    g->graph_prec.resize(n);
    for (int i = 0; i < n; ++i) {
      g->graph_P[i] = g->hs[i]->P;
      g->graph_rm[i] = g->hs[i]->maxrm;
      g->graph_prec[i] = g->hs[i]->precision;
    }
  }
  auto t0 = std::chrono::steady_clock::now();
  for (int w = 0; w < sweeps; ++w) KDQ_GCUDA(g, cudaGraphLaunch(g->graph, g->stream));
  // later work on each handle's own stream runs after the group's sweeps
  KDQ_GCUDA(g, cudaEventRecord(g->done, g->stream));
  for (int i = 0; i < n; ++i) {
    kdq_handle* h = g->hs[i];
    KDQ_GCUDA(g, cudaStreamWaitEvent(h->stream, g->done, 0));
    if (record) h->obs_rows += sweeps;
    h->last_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  return KDQ_OK;
}

int kdq_group_synchronize(kdq_group* g) {
  if (!g) return KDQ_ERR_ARG;
  KDQ_GCUDA(g, cudaSetDevice(g->device));
  KDQ_GCUDA(g, cudaStreamSynchronize(g->stream));
  for (size_t i = 0; i < g->hs.size(); ++i)
    if (int rc = kdq_synchronize(g->hs[i])) return gfail(g, rc, "handle " + std::to_string(i) + ": " + g->hs[i]->err);
  return KDQ_OK;
}

}  // extern "C"

namespace kdq {
// Message returned by kdq_last_error(NULL) for the handle-free entry points.
void set_global_error(const std::string& msg) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_create_err = msg;
}

size_t grover_scratch_bytes(int nA, int npairs, bool g_complex) {
  return (size_t)npairs * 3 * nA * nA * (g_complex ? 16 : 8);
}
}  // namespace kdq
