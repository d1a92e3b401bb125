"""Mixed-precision sweep (FP32 bulk products and updates, FP64 ratios and
stabilisation) against the FP64 oracle and against the FP64 sweep.

The FP32 Green's function is accurate to ~1e-6, so an acceptance test that
lands within that distance of its threshold can go the other way; on the
seeded cases below every decision coincides with the FP64 oracle's and G
agrees to 1e-4.  The measurements multiply G by products of up to a block of
slice matrices in FP32, whose condition number amplifies FP32 rounding to
~1e-4..1e-3 relative: far below the statistical error of any run, which is
what the last test checks (independent mixed and FP64 chains agree on the
mean energy within three standard errors).  Mixed precision exists for the
complex sweeps only: their HS factors are unitary (the real factors of t-V
are rejected).
"""
import numpy as np
import pytest

import cases
import dqmc_oracle as O
import philox
from kapdqmc_gb300 import Initial_s
from kapdqmc_gb300.sweep import Sweeper

pytestmark = pytest.mark.gpu

G_TOL, OBS_TOL, DRIFT_MAX = 1e-4, 2e-3, 1e-3


def _oracle(model, s, seed, chain, sweeps):
    n = O.proposals_per_sweep(model)
    ks, us = zip(*(philox.tape(seed, chain, w, n) for w in range(sweeps)))
    return O.phy_update(model, s, sweeps, O.Tape(np.concatenate(ks), np.concatenate(us)), True)


@pytest.mark.parametrize("make", [cases.tu_square, cases.tu_honeycomb, cases.tu_quench,
                                  cases.tuv_honeycomb, cases.tuv_square])
def test_mixed_tracks_fp64_oracle(make):
    model = make()
    nch, sweeps, seed = 2, 2, 77
    fields = np.stack([Initial_s(model, 300 + c) for c in range(nch)])
    n = O.proposals_per_sweep(model) * sweeps
    with Sweeper(model, nch) as sw:
        sw.set_precision("mixed")
        sw.set_fields(fields)
        sw.set_rng(seed)
        sw.enable_accept_log(n)
        obs = sw.phy_update(sweeps, 2)
        acc = sw.accept_log()
        s_gpu = sw.get_fields()
        G = [sw.green(c) for c in range(nch)]
        drift = sw.drift(sweeps)
    for c in range(nch):
        ref = _oracle(model, fields[c], seed, c, sweeps)
        np.testing.assert_array_equal(acc[c].astype(bool), np.array(ref.accepts))
        np.testing.assert_array_equal(s_gpu[c], ref.s)
        assert np.linalg.norm(G[c] - ref.G) / np.linalg.norm(ref.G) < G_TOL
        ro = np.array(ref.obs_rows)
        assert np.abs(obs[c] - ro).max() / max(1.0, np.abs(ro).max()) < OBS_TOL
        assert drift[c].max() < DRIFT_MAX


def test_mixed_rejected_for_real_hs_factors():
    from kapdqmc_gb300._lib import KdqError
    for model in (cases.tv_honeycomb(), cases.tuv_honeycomb(U=-4.0, V=0.3)):
        with Sweeper(model, 1) as sw:
            with pytest.raises(KdqError, match="unitary"):
                sw.set_precision("mixed")


@pytest.mark.parametrize("name", ["c3", "c4", "c5"])
def test_mixed_drift_at_config_sizes(name):
    model = getattr(cases, name)()
    with Sweeper(model, 4) as sw:
        sw.set_precision("mixed")
        sw.set_fields(np.stack([Initial_s(model, c) for c in range(4)]))
        sw.set_rng(5)
        sw.phy_update(1, 2)
        d = sw.drift(1)
    assert d.max() < DRIFT_MAX, d.max()


def test_mixed_energy_within_error_bars_of_fp64():
    model = cases.tu_honeycomb()
    nch, sweeps, burn = 128, 30, 5
    means = {}
    for prec, seed in (("fp64", 1), ("mixed", 2)):
        with Sweeper(model, nch) as sw:
            sw.set_precision(prec)
            sw.set_fields(np.stack([Initial_s(model, 1000 * seed + c) for c in range(nch)]))
            sw.set_rng(seed)
            obs = sw.phy_update(burn + sweeps, 2)
        ek = obs[:, burn:, 0].mean(axis=1)          # one mean per chain
        means[prec] = (ek.mean(), ek.std(ddof=1) / np.sqrt(nch))
    (m1, e1), (m2, e2) = means["fp64"], means["mixed"]
    assert abs(m1 - m2) < 3 * np.hypot(e1, e2), means


def _cholesky_pivot_ratios(model, s):
    """min_k R_kk^2 / max_k W_kk of the Cholesky W = R^H R of W = Z Z^H for the
    init chain's block products Z = BL_{k+1} BM_k (the mixed sweep's Cholesky
    QR rejects a block when this falls to 1e-8)."""
    sw = O._TUSweep(model, s, O.Tape(np.zeros(1, np.uint8), np.zeros(1)), False)
    sw.init_chain()
    out = []
    for idx in range(sw.NN - 1, 0, -1):
        Z = sw.BLs[idx + 1] @ sw.BM(idx)
        W = Z @ Z.conj().T
        try:
            R = np.linalg.cholesky(W)
        except np.linalg.LinAlgError:      # not positive definite in FP64 either
            out.append(0.0)
            continue
        out.append(float(np.min(np.abs(np.diag(R)) ** 2) / np.max(np.real(np.diag(W)))))
    return np.array(out)


def test_mixed_falls_back_to_householder_for_ill_conditioned_blocks():
    """dt = 0.5 and n_wrap = 10 on the 4x4 square lattice make the block
    products so ill-conditioned that the mixed sweep's Cholesky QR rejects
    them (pivot ratio below 1e-8, checked here on the oracle's blocks) and the
    Householder form runs.  FP32 wraps are too coarse to follow the FP64
    oracle's decisions at this dt (each slice's eK has condition number e^4),
    so the check is on the stabilisation itself: after the sweep, G at
    tau = 0 is recomputed from the chain's stabilised B-chains, and it must
    equal the oracle's G built from the same final fields, to the ~3e-3 that
    FP32 block products through such slices allow (1e-4 at the configured
    dt, test_mixed_tracks_fp64_oracle)."""
    from kapdqmc_gb300 import tU_Hubbard_Para
    model = tU_Hubbard_Para(Ht=1.0, Hu1=4.0, Hu2=4.0, Δt=0.5, Θrelax=5.0, Θquench=0.0,
                            Lattice="SQUARE45", site=[2, 4], BatchSize=10, Initial="H0")
    nch = 2
    fields = np.stack([Initial_s(model, 310 + c) for c in range(nch)])
    assert np.any(_cholesky_pivot_ratios(model, fields[0]) < 1e-8)
    with Sweeper(model, nch) as sw:
        sw.set_precision("mixed")
        sw.set_fields(fields)
        sw.set_rng(78)
        sw.phy_update(1, 0)
        s_end = sw.get_fields()
        G = [sw.green(c) for c in range(nch)]
    for c in range(nch):
        ref = O._TUSweep(model, s_end[c], O.Tape(np.zeros(1, np.uint8), np.zeros(1)), False)
        ref.init_chain()
        err = np.linalg.norm(G[c] - ref.G) / np.linalg.norm(ref.G)
        assert err < 1e-2, err
