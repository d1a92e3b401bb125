/*
 * kapdqmc.h — C ABI of libkapdqmc_gpu.so, the GB300 (sm_103a) projector-DQMC
 * sweep for KAPDQMC's t-U, t-V and t-UV models.
 *
 * The reference exposes the sweep as Julia methods; each entry point below
 * names the reference interface it replaces (paths are inside the KAPDQMC
 * project).  A Julia wrapper calls these through `ccall`; arrays are passed
 * in Julia's column-major layout, complex numbers as interleaved (re, im)
 * doubles.  Plain pointers and sizes only: the caller owns every host
 * array, the library copies what it needs during the call and keeps no host
 * pointer.  The library owns all device memory of a handle.
 *
 * Every function returns KDQ_OK (0) or a KDQ_ERR_* code; the message of the
 * last failure of a handle is returned by kdq_last_error().  A handle is not
 * thread-safe; distinct handles may be used from distinct threads.
 */
#ifndef KAPDQMC_H
#define KAPDQMC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  KDQ_OK = 0,
  KDQ_ERR_ARG = 1,      /* invalid argument or size (reference: @assert / error()) */
  KDQ_ERR_CUDA = 2,     /* CUDA runtime failure */
  KDQ_ERR_NUMERIC = 3,  /* NaN/Inf ratio, singular pivot, or drift above limit */
  KDQ_ERR_STATE = 4,    /* call out of order (e.g. tape exhausted) */
  KDQ_ERR_NOGPU = 5     /* no usable CUDA device */
};

enum { KDQ_TU = 0, KDQ_TV = 1, KDQ_TUV = 2 };

enum { KDQ_PREC_FP64 = 0, KDQ_PREC_MIXED = 1 };

enum { KDQ_SQUARE45 = 0, KDQ_SQUARE90 = 1, KDQ_HONEYCOMB120 = 2, KDQ_HONEYCOMB60 = 3 };

/* Model description: the fields of tU_Hubbard_Para_ / tV_Hubbard_Para_ /
 * tUV_Hubbard_Para_ that the sweep reads (src/tU/model.jl:14-37,
 * src/tV/model.jl:3-28, src/tUV/model.jl:3-27).  Matrices are Ns x Ns
 * column-major; Pt is Ns x Ns/2.  eK, eKinv, HalfeK, HalfeKinv and K are
 * complex (interleaved) iff k_complex; Pt is complex iff g_complex. */
typedef struct kdq_model_desc {
  int32_t kind;        /* KDQ_TU, KDQ_TV or KDQ_TUV */
  int32_t lattice;     /* KDQ_SQUARE45 ... KDQ_HONEYCOMB60 */
  int32_t site[2];     /* unit cells per direction */
  int32_t Ns;          /* sites (even) */
  int32_t Nt;          /* imaginary-time slices */
  int32_t z;           /* bond directions (tV, tUV); 1 for tU */
  int32_t g_complex;   /* sweep arithmetic: 1 complex128, 0 float64 */
  int32_t k_complex;   /* 1 if the kinetic matrices carry imaginary parts */
  int32_t n_nodes;     /* length of nodes */
  const int64_t* nodes;/* stabilisation nodes, 0 = nodes[0] < ... = Nt */
  const double* alpha; /* Nt coupling per slice (tU, tV); may be NULL for tUV */
  const double* gamma; /* 4 HS weights */
  const double* eta;   /* 4 HS fields */
  double a;            /* tUV: weight of a bond's second site */
  double Ht;           /* hopping */
  double U;            /* tUV interaction U (energy prefactor) */
  double V;            /* tUV interaction V (energy prefactor) */
  const double* eK;
  const double* eKinv;
  const double* HalfeK;
  const double* HalfeKinv;
  const double* K;
  const double* Pt;
  const int32_t* bonds;/* 1-based (x, y) pairs in nnidx's column-major order:
                          tV (Ns/2)*z pairs, tUV Ns*z pairs, NULL for tU */
} kdq_model_desc;

typedef struct kdq_handle kdq_handle;

typedef struct kdq_stats {
  int64_t proposals;   /* proposals made by all chains in the last call */
  int64_t accepted;    /* accepted proposals */
  int64_t recomputes;  /* stabilisation recomputes of G */
  double max_drift;    /* max ||G_wrap - G_recompute||_F / ||G_recompute||_F */
  double seconds;      /* wall time of the last kdq_phy_update / kdq_sweep */
} kdq_stats;

/* Create a handle with n_chains independent Markov chains of one model on a
 * CUDA device, uploading the model (replaces the per-call buffer set-up of
 * phy_update: PhyBuffer, src/tU/model.jl:151-165; src/public/Buffer.jl:3-19). */
int kdq_create(kdq_handle** out, const kdq_model_desc* model, int32_t n_chains, int32_t device);

/* Free all device memory of the handle. */
void kdq_destroy(kdq_handle* h);

/* Message of the last failure on h (or of the last kdq_create failure when
 * h is NULL).  Valid until the next call on h. */
const char* kdq_last_error(const kdq_handle* h);

/* HS fields of all chains: n_chains consecutive arrays, each in the layout of
 * the reference's `s` (tU: Ns x Nt, src/tU/GreenMatrix.jl:1-8; tV:
 * (Ns/2) x z x Nt, src/tV/GreenMatrix.jl:1-10; tUV: Ns*z x Nt,
 * src/tUV/GreenMatrix.jl:1-8), values in {1,2,3,4}.  nbytes must equal
 * n_chains * Nt * n_field. */
int kdq_set_fields(kdq_handle* h, const uint8_t* s, size_t nbytes);
int kdq_get_fields(kdq_handle* h, uint8_t* s, size_t nbytes);

/* Random stream: Philox4x32-10, key = seed, counter = (proposal index in
 * sweep, sweep index, chain, stream id).  sweep_offset is the sweep index of
 * the next sweep; it advances by one per sweep.  Replaces the reference's
 * unseedable MersenneTwister(threadid()+time_ns()) (src/tU/phy_update.jl:31). */
int kdq_set_rng(kdq_handle* h, uint64_t seed, uint64_t sweep_offset);

/* Explicit proposal tape in the reference's consumption order
 * (src/tU/phy_update.jl:259,262): per proposal a choice index k in {0,1,2}
 * among the three values other than the current one (ascending) and a
 * uniform u in [0,1).  n_per_chain entries per chain, chain-major.  The next
 * kdq_phy_update/kdq_sweep consumes it from its start; a tape shorter than
 * the sweeps need fails with KDQ_ERR_STATE.  kdq_set_rng switches back to
 * the Philox stream. */
int kdq_set_tape(kdq_handle* h, const uint8_t* k, const double* u, size_t n_per_chain);

/* The reference's phy_update(path, model, s, Sweeps, record) for all chains:
 * rebuild the left B chain and G from the current fields, run `sweeps`
 * forward+backward sweeps with local updates and QR stabilisation, and
 * return the per-sweep measurement rows when record != 0 (tU: Ek Eu CDW0
 * CDW1 SDW0 SDW1; tV: Ek Ev R0[4] R1[4]; tUV: Ek Eu Ev CDW0 CDW1 SDW0 SDW1).
 * record = 1 measures exactly as the reference (a copy of G wrapped slice by
 * slice to Nt/2 for every measured slice); record = 2 gives the same
 * estimator with the wraps folded into two products L, R kept between
 * measurements (G0 = L G R; same observables up to rounding, far fewer
 * GEMMs).  obs may be NULL when record == 0; otherwise obs_len must be at least
 * n_chains * sweeps * kdq_n_obs(h), filled chain-major.
 * Replaces src/tU/phy_update.jl:3-152, src/tV/phy_update.jl:1-188,
 * src/tUV/phy_update.jl:1-186 (the CSV append is left to the caller). */
int kdq_phy_update(kdq_handle* h, int32_t sweeps, int32_t record, double* obs, size_t obs_len);

/* Split form of kdq_phy_update for callers that keep the state resident:
 * kdq_init rebuilds the B chain and G from the current fields
 * (src/tU/phy_update.jl:39-50); kdq_sweep continues from the current state
 * without host copies (asynchronous on the handle's stream; observables stay
 * on the device until kdq_get_obs). */
int kdq_init(kdq_handle* h);
int kdq_sweep(kdq_handle* h, int32_t sweeps, int32_t record);
int kdq_get_obs(kdq_handle* h, double* obs, size_t obs_len);
int kdq_synchronize(kdq_handle* h);

/* t-U and complex t-UV: append 4 columns to every measurement row, making
 * 10 (t-U) or 11 (t-UV); 0 restores the reference's 6 or 7.  Honeycomb
 * lattices: the structure factors CDW0, CDW1, SDW0, SDW1 with all terms of
 * each correlator (the reference's columns keep only the first term: its
 * `+adjoint(...)` continuation lines are discarded statements,
 * src/tU/phy_update.jl:194-235, src/tUV/phy_update.jl:306-323).  Square
 * lattices (where the reference measures no structure factor): the
 * staggered charge structure factor at (pi, pi), 0, the staggered spin
 * structure factor at (pi, pi), 0, i.e. sum_ij e_i e_j <rho_i rho_j> / Ns^2
 * with e the lattice's two-colouring.  Drops rows recorded so far.  No
 * counterpart in the reference. */
int kdq_set_measure_full(kdq_handle* h, int32_t enable);

/* Number of measurement columns per sweep row (6, 10 or 7). */
int kdq_n_obs(const kdq_handle* h);

/* Equal-time Green's function of one chain at the current slice (Ns x Ns,
 * column-major, interleaved complex iff g_complex).  len counts doubles. */
int kdq_get_green(kdq_handle* h, int32_t chain, double* G, size_t len);

/* Statistics of the last kdq_phy_update / kdq_sweep call. */
int kdq_get_stats(kdq_handle* h, kdq_stats* st);

/* Log-weight of each chain's current fields: logdet[c] = log|det(P^H B(Theta,0) P)|
 * with B(Theta,0) the product of all slice matrices, and phase[2c], phase[2c+1]
 * = det/|det| (re, im), as of the last G recompute (the end of kdq_init and of
 * every sweep).  The stabilised B chains keep the log|det| of the triangular
 * factors the QR steps drop; the reference discards them (src/tU/phy_update.jl:
 * 85-86,133-134), so this has no counterpart there.  The full configuration
 * weight adds the local factors: t-U and complex t-UV |det|^2 prod gamma, t-V
 * det prod gamma, real t-UV det^2 prod gamma e^{-(a+1) eta}
 * (the ratios of src/tU/phy_update.jl:261, src/tV/phy_update.jl:196-199,
 * src/tUV/phy_update.jl:192-197).  len counts chains. */
int kdq_get_log_det(kdq_handle* h, double* logdet, double* phase, size_t len);

/* Debug record of accept decisions (1 byte per proposal, chain-major, in
 * tape order) of the next calls; enable before kdq_phy_update.  Replaces the
 * reference's commented-out checks (src/tV/phy_update.jl:74-90). */
int kdq_enable_accept_log(kdq_handle* h, size_t n_per_chain);
int kdq_get_accept_log(kdq_handle* h, uint8_t* flags, size_t nbytes);

/* Drift ||G_wrap - G_recompute||_F / ||G_recompute||_F at every recompute of
 * the last call, chain-major, 2*(n_nodes-1) per sweep (the reference's
 * "Batchsize Wrap Error" check, src/tU/phy_update.jl:89-97). */
int kdq_get_drift(kdq_handle* h, double* drift, size_t len);

/* Swap-replica Rényi-2 Grover determinant det(2 G1_A G2_A - G1_A - G2_A + I)
 * (GroverMatrix!, src/public/GF.jl:101-109, and the det of get_ABGM!,
 * src/tU/SCEE.jl:264-276) for npairs replica pairs.  G holds 2*npairs
 * Ns x Ns matrices (pair p = matrices 2p and 2p+1; host memory, column-major,
 * interleaved complex iff g_complex); index holds the nA 1-based sites of
 * region A; det receives (re, im) per pair.  e^{-S2} is estimated by
 * <|det|^2> for the spinful models and <det> for t-V. */
int kdq_grover_det(const double* G, int32_t Ns, int32_t g_complex, int32_t npairs, const int32_t* index,
                   int32_t nA, double* det, int32_t device);

/* The same for the chains of a handle, paired (0,1), (2,3), ..., at their
 * current time slice. */
int kdq_grover_det_chains(kdq_handle* h, const int32_t* index, int32_t nA, double* det);

/* Keep a copy of every chain's equal-time G at the middle slice tau = Nt/2
 * (the G0 of the reference's G4!, src/public/Gupdate.jl:159-212) whenever a
 * recording sweep passes it, and evaluate the Grover determinant of the chain
 * pairs (0,1), (2,3), ... on those copies: the independent-replica estimator
 * of e^{-S2} at the middle of the projection. */
int kdq_keep_middle_green(kdq_handle* h, int32_t enable);
int kdq_grover_det_middle(kdq_handle* h, const int32_t* index, int32_t nA, double* det);

/* Allocation-free form of kdq_grover_det, for callers that must not call
 * cudaMalloc (work recorded into a CUDA graph or run where a device
 * synchronisation is unaffordable, and processes whose free device memory is
 * held by another allocator).  No counterpart in the reference.  G (2*npairs
 * Ns x Ns matrices), index (nA 1-based sites) and det (2*npairs doubles) are
 * DEVICE pointers supplied by the caller; the work is queued on `stream`
 * (a cudaStream_t; NULL = default stream) and det is valid once that stream
 * has been synchronised.  Scratch comes from one fixed 8 MiB device array per
 * GPU, shared by all calls: requests needing more (npairs * (3 nA^2 elements
 * + nA ints) plus nA ints, with 256-byte padding) fail with KDQ_ERR_ARG, and
 * calls that overlap on the GPU race on the array.  Region indices outside
 * 1..Ns give NaN determinants.  Every call whose stream is not capturing
 * looks up the array's device address (again after a cudaDeviceReset, which
 * can move it); a call inside a stream capture reuses the address of the
 * device's last uncaptured call, so make the first call on a device before
 * any stream capture, and one more after a cudaDeviceReset.  Errors are
 * reported through kdq_last_error(NULL). */
int kdq_grover_det_noalloc(const double* G, int32_t Ns, int32_t g_complex, int32_t npairs,
                           const int32_t* index, int32_t nA, double* det, void* stream);

/* Arithmetic of the sweep.  KDQ_PREC_FP64 (default): everything in FP64, the
 * reference's arithmetic.  KDQ_PREC_MIXED: G is held in FP32; the products
 * with a real kinetic matrix (slice wraps, block products of the
 * stabilisation chain, the measurement's kinetic factors) run as 3xTF32
 * tensor-core tiles with FP32 accumulation (FP32 CUDA-core products when
 * the hopping is complex), the rank-k updates of G in FP32, delayed and
 * applied in batches of up to 16 vectors (complex G: as 3xTF32 tensor-core
 * products); the acceptance ratios stay FP64; the thin QR (Cholesky QR,
 * Householder when a block is ill-conditioned), BL BR and its inverse at
 * every node run in double-float arithmetic (two FP32 values, 48-bit
 * significand, ~1e-14 relative), and the two products that form the FP32 G
 * from them, (BL BR)^-1 BL and BR X, as 3xTF32 tensor-core products (complex
 * G); kdq_get_drift then reports ||G_FP32-wrap - G_recompute||_F / ||G||_F.
 * Only the complex sweeps
 * (t-U, t-UV with U > 0) accept it: their HS factors cis(alpha eta) are
 * unitary, while the real factors exp(+-alpha eta) of t-V and real t-UV
 * amplify FP32 rounding in the wraps (KDQ_ERR_ARG).  No counterpart in the
 * reference (which is FP64 only).  Call before kdq_init / kdq_phy_update. */
int kdq_set_precision(kdq_handle* h, int32_t mode);

/* Per-stage clock counts of the sweep (SM clock cycles, summed over chains):
 * cycles[0] wraps, [1] local updates (FP64 sweep: the windows of
 * acceptance ratios and the G updates of accepted proposals; mixed sweep:
 * the accepted proposals' update vectors and the flushes of the delayed
 * updates), [2] measurements, [3] block products of the stabilisation chain,
 * [4] QR, [5] G recompute, [6] self-learning cluster moves, [7] the mixed
 * sweep's windows of acceptance ratios; cycles has 8 entries.  Enabling resets the counters and adds a barrier
 * per stage.  No counterpart in the reference (which has no tracing). */
int kdq_enable_phase_timing(kdq_handle* h, int32_t enable);
int kdq_get_phase_cycles(kdq_handle* h, double* cycles);

/* Replay each sweep's launches (see kdq_set_sweep_launch) from a captured
 * CUDA graph (default on) or launch them one by one (enable = 0).  The graph is
 * re-captured whenever the launch parameters change.  No counterpart in the
 * reference (a launch-sequencing choice of this implementation). */
int kdq_set_graphs(kdq_handle* h, int32_t enable);

/* Launch shape of a sweep: 0 (default) one launch per stabilisation block,
 * 2 (NN-1) per sweep; 1 one launch in which every chain's CTA runs all of
 * the sweep's blocks (chains are independent, so no CTA waits for another
 * between blocks; measured 2 % slower on t-U 12x12 with 256 chains).
 * Results are identical.  No counterpart in the reference. */
int kdq_set_sweep_launch(kdq_handle* h, int32_t per_sweep);

/* CUDA stream (cudaStream_t) of the handle, for event timing by callers. */
void* kdq_stream(kdq_handle* h);

/* Register-tile class of the sweep kernel: rows = 1, 3 or 6 row groups of
 * 32 sites, at least ceil(Ns / 32) (the default is the smallest class that
 * fits).  Every class computes the same arithmetic in the same order, so the
 * choice changes speed only.  kdq_get_tiles returns the current class.
 * kdq_autotune times one sweep of the handle's own chains per valid class,
 * keeps the fastest, puts the fields and each chain's random-stream position
 * back and leaves the handle as kdq_init does; ms[0..2] receive the sweep
 * times of classes 1, 3, 6 (-1 where a class does not fit).  On failure the
 * fields and positions are put back and kdq_init must run again.  Choices are
 * cached per device, model, size, precision and batch for the process.  No
 * counterpart in the reference (which calls BLAS). */
int kdq_set_tiles(kdq_handle* h, int32_t rows);
int kdq_get_tiles(const kdq_handle* h);
int kdq_autotune(kdq_handle* h, int32_t* chosen, double* ms, int32_t len);

/* Groups: handles of different lattices, models or precisions on one device
 * swept together.  kdq_group_sweep runs `sweeps` sweeps of every handle of
 * the group (each initialised by kdq_init) as one CUDA graph per sweep whose
 * parallel branches are the handles' block launches; results are those of
 * kdq_sweep on each handle alone (same kernels, same random streams).
 * kdq_group_synchronize waits and checks every handle's error flags;
 * kdq_get_obs and the other per-handle calls read the results.  A handle
 * may belong to several groups but must not be used from another thread
 * during a group call, and a group must be destroyed before its handles.
 * The group always replays a captured graph (kdq_set_graphs does not
 * apply).  Reference counterpart: none (the reference runs one
 * model per Julia call, src/tU/phy_update.jl:3). */
typedef struct kdq_group kdq_group;
int kdq_group_create(kdq_group** out, kdq_handle* const* handles, int32_t n);
int kdq_group_sweep(kdq_group* g, int32_t sweeps, int32_t record);
int kdq_group_synchronize(kdq_group* g);
const char* kdq_group_last_error(const kdq_group* g);
void kdq_group_destroy(kdq_group* g);

/* ---------------------------------------------------------------------
 * Self-learning Monte Carlo (t-U).  No counterpart in the reference, which
 * has local updates only (src/tU/phy_update.jl:256-267).
 *
 * Effective model: a periodic three-layer convolutional net (16 channels,
 * 3x3 kernels, tanh) over the slice x site field s (Nt rows of Ns sites; a
 * configuration is laid out as the sweep's fields, s[t * Ns + i] in 1..4),
 * whose output summed over all positions, F(s), is fitted to the fermion part
 * 2 log|det(P^H B(Theta,0) P)| of the log-weight (kdq_get_log_det).
 * params: KDQ_CNN_NPARAM floats, in the order W1[16][4][3][3] (one-hot
 * input channels), b1[16], W2[16][16][3][3], b2[16], W3[1][16][3][3], b3;
 * the kernels compute with the bf16-rounded weights and FP32 accumulation.
 * The three calls below are handle-free; errors go to kdq_last_error(NULL). */
#define KDQ_CNN_PARAMS 3057

/* F(s_b) of n_cfg configurations. */
int kdq_cnn_forward(const uint8_t* fields, int32_t n_cfg, int32_t Nt, int32_t Ns, const float* params,
                    double* F, int32_t device);

/* Gradient of sum_b dF[b] F(s_b) with respect to params (KDQ_CNN_PARAMS floats). */
int kdq_cnn_grad(const uint8_t* fields, const double* dF, int32_t n_cfg, int32_t Nt, int32_t Ns,
                 const float* params, float* grad, int32_t device);

/* Fits F to target[b] by minimising the mean squared error with Adam
 * (beta 0.9, 0.999, eps 1e-8, learning rate lr) over `epochs` passes in
 * shuffled mini-batches of `batch` configurations (shuffle seeded by seed);
 * params is updated in place and loss_per_epoch (epochs doubles, may be NULL)
 * receives each epoch's squared error averaged over its batches, each batch
 * measured before its own update. */
int kdq_cnn_train(const uint8_t* fields, const double* target, int32_t n_cfg, int32_t Nt, int32_t Ns,
                  int32_t epochs, int32_t batch, float lr, uint64_t seed, float* params,
                  double* loss_per_epoch, int32_t device);

/* Self-learning cluster moves in the t-U sweep.  After the local updates of
 * every slice (both sweep directions) the sweep makes moves_per_slice moves:
 * each picks cluster_len consecutive sites of the slice (random start, sites
 * mod Ns), runs eff_steps single-site Metropolis steps on the effective
 * weight exp(F(s)) prod gamma[s] of the model `params` (KDQ_CNN_PARAMS floats,
 * evaluated incrementally in FP32 with bf16 weights), and accepts the changed
 * sites S together with probability min(1, |det(I + Delta_S (I - G_SS))|^2
 * exp(-(F(s') - F(s)))), the exact FP64 ratio of the full weight over the
 * effective one; G then takes the rank-|S| form of Gupdate!
 * (src/public/Gupdate.jl:5-11).  Random numbers come from Philox4x32-10 on
 * the kdq_set_rng seed with a stream of their own, also when a tape is set.
 * moves_per_slice = 0 turns the moves off.  Needs cluster_len <= min(32,
 * Ns/2, Ns-8) and Nt >= 9. */
int kdq_slmc_enable(kdq_handle* h, const float* params, int32_t moves_per_slice, int32_t cluster_len,
                    int32_t eff_steps);

/* Coupled incremental SCEE sweep, ctrl_SCEEicr(path, model, indexA, indexB,
 * Sweeps, lambda, Nlambda, ss, record) (src/tU/SCEE.jl:1-211,
 * src/tV/SCEE.jl:1-431, src/tUV/SCEE.jl:1-339), t-U, t-V and t-UV in FP64.
 * Chains 2p and 2p+1 of the handle are the two replicas ss[1], ss[2] of pair
 * p (fields through kdq_set_fields, random stream through kdq_set_rng or
 * kdq_set_tape, replica r of pair p drawing from chain 2p+r's stream in the
 * plain sweep's order).  kdq_scee_enable sets the regions (1-based sites,
 * at most min(Ns/2, 96) each), lambda in [0,1] and Nlambda.  kdq_scee_run
 * builds every replica's block products and stabilised chains and runs
 * `sweeps` coupled sweeps: each site proposal of either replica is accepted
 * with its local ratio times |det g_A'/det g_A|^(2 lambda) |det g_B'/det g_B|^(2 (1-lambda))
 * (t-U, UpdateSCEELayer!, src/tU/SCEE.jl:230-287; t-V: each bond proposal
 * with (det g_A'/det g_A)^lambda (det g_B'/det g_B)^(1-lambda), the bond
 * rotations of each direction wrapped between that direction's updates,
 * src/tV/SCEE.jl:87-330,447-508; t-UV: bond proposals with
 * |det Tau|^2 factors and without the plain sweep's real-type factor,
 * src/tUV/SCEE.jl:355-402).  O receives per pair the reference's CSV
 * row: O[p (sweeps+1)] = lambda, then per sweep the mean over slices of
 * (detg_A / detg_B)^(1/Nlambda), detg = |det g|^2 (t-U, t-UV) or det g (t-V);
 * len counts doubles.  kdq_scee_get_green copies one replica's Green's
 * function `which` (0: G(tau,tau), 1: G(tau0,tau0) at the middle node,
 * 2: G(tau,tau0), 3: G(tau0,tau); Ns^2 values, complex sweeps as 2 doubles
 * each) at the end of the run (tau = 0).
 * After kdq_scee_run, kdq_init must precede a plain sweep. */
int kdq_scee_enable(kdq_handle* h, const int32_t* indexA, int32_t nA, const int32_t* indexB, int32_t nB,
                    double lambda, int32_t n_lambda);
int kdq_scee_run(kdq_handle* h, int32_t sweeps, double* O, size_t len);
int kdq_scee_get_green(kdq_handle* h, int32_t chain, int32_t which, double* G, size_t len);

/* Disorder-operator sweep ctrl_SCDOPicr(path, model, alpha, indexA, indexB,
 * Sweeps, lambda, Nlambda, s, record) (src/tU/disorder_operate.jl:1-247),
 * t-U in FP64: every chain runs on its own, its weight reweighted by
 * |det X_A|^(2 lambda) |det X_B|^(2 (1-lambda)) with
 * X = e^{i alpha} I + (1 - e^{i alpha}) G(tau0,tau0)[R,R].  O receives per
 * chain lambda, then per sweep the mean over slices of
 * (|det X_A|^2 / |det X_B|^2)^(1/Nlambda); kdq_scee_get_green reads the
 * chain's Green's functions afterwards. */
int kdq_dop_enable(kdq_handle* h, double alpha, const int32_t* indexA, int32_t nA, const int32_t* indexB,
                   int32_t nB, double lambda, int32_t n_lambda);
int kdq_dop_run(kdq_handle* h, int32_t sweeps, double* O, size_t len);

/* Cluster moves of the last kdq_phy_update / kdq_sweep call, summed over
 * chains: counts[0] proposed, counts[1] accepted, counts[2] proposals in
 * which the effective-model chain changed no site (accepted trivially, not
 * counted in counts[1]). */
int kdq_get_slmc_stats(kdq_handle* h, int64_t* counts);

#ifdef __cplusplus
}
#endif
#endif /* KAPDQMC_H */
