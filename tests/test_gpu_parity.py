"""Parity of the CUDA sweep (through the C ABI) with the CPU oracle.

Same model, same fields, same Philox proposal stream: the accept/reject
sequence and the final fields must be identical, G must agree to 1e-10
(relative Frobenius) and the measurement rows to 1e-9 (relative).
"""
import numpy as np
import pytest

import cases
import dqmc_oracle as O
import philox
from kapdqmc_gb300 import Initial_s
from kapdqmc_gb300.sweep import Sweeper

pytestmark = pytest.mark.gpu

G_TOL = 1e-10       # relative Frobenius distance of G
OBS_TOL = 1e-9      # relative distance of each measurement row


def _oracle(model, s, seed, chain, sweeps, record):
    n = O.proposals_per_sweep(model)
    ks, us = zip(*(philox.tape(seed, chain, w, n) for w in range(sweeps)))
    return O.phy_update(model, s, sweeps, O.Tape(np.concatenate(ks), np.concatenate(us)), record)


def _compare(model, nchains=2, sweeps=2, record=True, seed=1234, obs_tol=OBS_TOL):
    fields = np.stack([Initial_s(model, 100 + c) for c in range(nchains)])
    n = O.proposals_per_sweep(model) * sweeps
    with Sweeper(model, nchains) as sw:
        sw.set_fields(fields)
        sw.set_rng(seed)
        sw.enable_accept_log(n)
        obs = sw.phy_update(sweeps, record)
        s_gpu = sw.get_fields()
        acc = sw.accept_log()
        G = [sw.green(c) for c in range(nchains)]
        st = sw.stats()
        drift = sw.drift(sweeps)
    for c in range(nchains):
        ref = _oracle(model, fields[c], seed, c, sweeps, record)
        np.testing.assert_array_equal(acc[c].astype(bool), np.array(ref.accepts), err_msg=f"chain {c} accepts")
        np.testing.assert_array_equal(s_gpu[c], ref.s, err_msg=f"chain {c} fields")
        rel = np.linalg.norm(G[c] - ref.G) / np.linalg.norm(ref.G)
        assert rel < G_TOL, f"chain {c}: G rel diff {rel:.3e}"
        if record:
            ro = np.array(ref.obs_rows)
            err = np.abs(obs[c] - ro).max() / max(1.0, np.abs(ro).max())
            assert err < obs_tol, f"chain {c}: obs diff {err:.3e}\n{obs[c]}\n{ro}"
        # the drift measures the rounding accumulated by the wraps between two
        # recomputes; the two implementations round differently, so their drift
        # values agree in magnitude, not digit by digit
        rd = np.array(ref.drift)
        assert np.all(drift[c] <= np.maximum(10 * rd, 1e-8)) and np.all(rd <= np.maximum(10 * drift[c], 1e-8)), \
            f"chain {c}: drift {drift[c].max():.2e} vs {rd.max():.2e}"
        assert drift[c].max() < 1e-5
    assert st["proposals"] == nchains * n
    assert st["max_drift"] < 1e-6
    return st


def test_tu_square():
    _compare(cases.tu_square())


def test_tu_honeycomb_structure_factors():
    _compare(cases.tu_honeycomb())


def test_tu_quench_ragged_nodes():
    # quench profile (slice-dependent α) and the reference's own test model
    _compare(cases.tu_quench(), sweeps=1)


def test_tu_flux_complex_kinetic():
    _compare(cases.tu_square(flux=np.pi), record=False)


@pytest.mark.parametrize("make", [cases.tu_square90_flux, cases.tu_honeycomb60, cases.tv_honeycomb60,
                                  cases.tuv_honeycomb60])
def test_other_lattices(make):
    # SQUARE90 with pi flux (complex hopping) and the HoneyComb60 geometry
    _compare(make(), record=False)


def test_tv_honeycomb():
    _compare(cases.tv_honeycomb())


def test_tuv_honeycomb_complex():
    _compare(cases.tuv_honeycomb())


def test_tuv_honeycomb_real():
    _compare(cases.tuv_honeycomb(U=-4.0, V=0.3))


def test_tuv_square_marginal():
    _compare(cases.tuv_square())


def test_c1_config_one_sweep():
    # t-U 4x4, 100 slices, n_wrap 10: the single-chain configuration
    _compare(cases.c1(), nchains=1, sweeps=1)


def test_explicit_tape_matches_philox():
    model = cases.tu_square()
    s0 = Initial_s(model, 5)
    n = O.proposals_per_sweep(model)
    k, u = philox.tape(99, 0, 0, n)
    with Sweeper(model, 1) as sw:
        sw.set_fields(s0)
        sw.set_rng(99)
        sw.phy_update(1)
        a = sw.get_fields()
        sw.set_fields(s0)
        sw.set_tape(k[None], u[None])
        sw.phy_update(1)
        b = sw.get_fields()
    np.testing.assert_array_equal(a, b)


def test_tape_too_short_is_an_error():
    from kapdqmc_gb300._lib import KdqError
    model = cases.tu_square()
    n = O.proposals_per_sweep(model)
    with Sweeper(model, 1) as sw:
        sw.set_fields(Initial_s(model, 5))
        sw.set_tape(np.zeros((1, n - 1)), np.full((1, n - 1), 0.5))
        with pytest.raises(KdqError):
            sw.phy_update(1)


def test_split_api_continues_state():
    """init + sweep(1) + sweep(1) equals phy_update(2) on the same stream."""
    model = cases.tv_honeycomb()
    s0 = np.stack([Initial_s(model, 7), Initial_s(model, 8)])
    with Sweeper(model, 2) as sw:
        sw.set_fields(s0)
        sw.set_rng(5)
        o2 = sw.phy_update(2, True)
        g2 = sw.get_fields()
        sw.set_fields(s0)
        sw.set_rng(5)
        sw.init()
        sw.sweep(1, True)
        sw.sweep(1, True)
        sw.synchronize()
        o11 = sw.get_obs(2)
        g11 = sw.get_fields()
    np.testing.assert_array_equal(g2, g11)
    np.testing.assert_allclose(o2, o11, rtol=1e-12, atol=0)


@pytest.mark.parametrize("cplx", [True, False])
def test_grover_det_matches_oracle(cplx):
    from kapdqmc_gb300.sweep import grover_det
    rng = np.random.default_rng(3)
    Ns, npairs = 64, 5
    index = list(range(1, 33))                     # region A = 32 sites
    Gs = []
    for _ in range(2 * npairs):
        A = rng.normal(size=(Ns, Ns // 2)) + (1j * rng.normal(size=(Ns, Ns // 2)) if cplx else 0)
        Q = np.linalg.qr(A)[0]
        Gs.append(np.eye(Ns) - Q @ Q.conj().T)    # a pure-state Green's function
    G1, G2 = np.array(Gs[0::2]), np.array(Gs[1::2])
    got = grover_det(G1, G2, index)
    want = np.array([O.grover_det(a, b, index) for a, b in zip(G1, G2)])
    np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-14)


def test_grover_det_of_sweep_chains():
    model = cases.tuv_square()
    fields = np.stack([Initial_s(model, 40 + c) for c in range(4)])
    index = list(range(1, 9))
    with Sweeper(model, 4) as sw:
        sw.set_fields(fields)
        sw.set_rng(11)
        sw.phy_update(1)
        dets = sw.grover_det(index)
        G = [sw.green(c) for c in range(4)]
    want = [O.grover_det(G[0], G[1], index), O.grover_det(G[2], G[3], index)]
    np.testing.assert_allclose(dets, want, rtol=1e-10, atol=1e-14)


# record = 2: the measurement wraps folded into the products L, R (reassociated
# arithmetic, same estimator): rows agree with the reference's to 1e-8.
FAST_TOL = 1e-8


@pytest.mark.parametrize("make", [cases.tu_square, cases.tu_honeycomb, cases.tu_quench, cases.tv_honeycomb,
                                  cases.tuv_honeycomb, cases.tuv_square])
def test_fast_measurement_matches_reference_window(make):
    _compare(make(), sweeps=3, record=2, obs_tol=FAST_TOL)


def test_fast_measurement_c1():
    _compare(cases.c1(), nchains=1, sweeps=2, record=2, obs_tol=FAST_TOL)


# The configurations themselves, one chain and one sweep each: these run the
# N <= 192 (six row groups), complex N = 64 and real N = 72 kernel variants.
@pytest.mark.parametrize("name", ["c2", "c3", "c4", "c5"])
def test_config_sizes_one_sweep(name):
    _compare(getattr(cases, name)(), nchains=1, sweeps=1, record=2, obs_tol=FAST_TOL)


def test_graph_replay_equals_direct_launches():
    model = cases.tv_honeycomb()
    s0 = np.stack([Initial_s(model, 70 + c) for c in range(3)])
    out = []
    for graphs in (True, False):
        with Sweeper(model, 3) as sw:
            sw.set_graphs(graphs)
            sw.set_fields(s0)
            sw.set_rng(9)
            o = sw.phy_update(3, 2)
            out.append((o, sw.get_fields(), sw.green(1), sw.drift(3)))
    np.testing.assert_array_equal(out[0][1], out[1][1])
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][2], out[1][2])
    np.testing.assert_array_equal(out[0][3], out[1][3])


def test_grover_det_at_middle_slice():
    """Pairs of chains on their G at tau = Nt/2, as the oracle holds it when the
    sweep passes the middle slice (the last pass is the backward one)."""
    model = cases.tuv_square()
    fields = np.stack([Initial_s(model, 60 + c) for c in range(4)])
    index = list(range(1, 9))
    seed = 13
    with Sweeper(model, 4) as sw:
        sw.keep_middle_green(True)
        sw.set_fields(fields)
        sw.set_rng(seed)
        sw.phy_update(1, 2)
        dets = sw.grover_det_middle(index)
    mids = []
    for c in range(4):
        n = O.proposals_per_sweep(model)
        k, u = philox.tape(seed, c, 0, n)
        sw_o = O._TUVSweep(model, fields[c], O.Tape(k, u), True)
        held = {}
        orig = sw_o.measure

        def grab(t0, _orig=orig, _held=held):
            if 2 * t0 == model.Nt:
                _held["G"] = sw_o.G.copy()
            return _orig(t0)
        sw_o.measure = grab
        sw_o.run(1)
        mids.append(held["G"])
    want = [O.grover_det(mids[0], mids[1], index), O.grover_det(mids[2], mids[3], index)]
    np.testing.assert_allclose(dets, want, rtol=1e-8, atol=1e-12)


@pytest.mark.parametrize("record", [1, 2])
@pytest.mark.parametrize("make,ncol", [(cases.tu_honeycomb, 10), (cases.tuv_honeycomb, 11),
                                      (cases.tu_square, 10), (cases.tuv_square, 11)])
def test_full_structure_factors(record, make, ncol):
    # honeycomb t-U and complex t-UV with the structure factors' discarded
    # adjoint terms restored (4 columns after the reference's); on the square
    # lattices the staggered (pi, pi) charge and spin structure factors
    model = make()
    nch, sweeps, seed = 2, 2, 77
    fields = np.stack([Initial_s(model, 300 + c) for c in range(nch)])
    with Sweeper(model, nch) as sw:
        sw.set_measure_full(True)
        sw.set_fields(fields)
        sw.set_rng(seed)
        obs = sw.phy_update(sweeps, record)
    assert obs.shape == (nch, sweeps, ncol)
    for c in range(nch):
        ref = _oracle_full(model, fields[c], seed, c, sweeps)
        ro = np.array(ref.obs_rows)
        err = np.abs(obs[c] - ro).max() / max(1.0, np.abs(ro).max())
        assert err < (1e-8 if record == 2 else 1e-9), err


def _oracle_full(model, s, seed, chain, sweeps):
    n = O.proposals_per_sweep(model)
    ks, us = zip(*(philox.tape(seed, chain, w, n) for w in range(sweeps)))
    return O.phy_update(model, s, sweeps, O.Tape(np.concatenate(ks), np.concatenate(us)), True, full_sf=True)
