"""Log-weights of HS configurations (CPU): the oracle's stabilised log|det|
against a direct determinant, and the full log-weight against the
acceptance ratios the sweep uses (src/tU/phy_update.jl:256-267,
src/tUV/phy_update.jl:188-203)."""
import numpy as np
import pytest

import cases
import dqmc_oracle as O
from kapdqmc_gb300 import Initial_s
from kapdqmc_gb300.sweep import log_weight


def _direct(model, s):
    sw = O._SWEEPS[model.kind](model, s, O.Tape([], []), False)
    B = np.eye(model.Ns, dtype=sw.dtype)
    for lt in range(1, model.Nt + 1):
        B = sw.B_left(lt, B)
    d = np.linalg.det(model.Pt.conj().T.astype(sw.dtype) @ B @ model.Pt.astype(sw.dtype))
    return np.log(abs(d)), d / abs(d)


@pytest.mark.parametrize("make", [cases.tu_square, cases.tu_honeycomb, cases.tv_honeycomb,
                                  cases.tuv_honeycomb, cases.tuv_square,
                                  lambda: cases.tuv_honeycomb(U=-4.0)])
def test_stabilised_log_det_matches_direct_determinant(make):
    model = make()
    s = Initial_s(model, 5)
    ld, ph = O.log_det(model, s)
    ld0, ph0 = _direct(model, s)
    assert abs(ld - ld0) < 1e-9 * max(1.0, abs(ld0))
    assert abs(ph - ph0) < 1e-9


def _ratio_tu(model, s, lt, i, sx):
    G = O.G_tau(model, s, lt)
    sold = int(s[i, lt - 1])
    Δ = np.exp(1j * model.α[lt - 1] * (model.η[sx - 1] - model.η[sold - 1])) - 1
    pc = 1 + Δ * (1 - G[i, i])
    return abs(pc) ** 2 * model.γ[sx - 1] / model.γ[sold - 1]


def _ratio_tuv(model, s, lt, b, sx):
    sw = O._TUVSweep(model, s, O.Tape([], []), False)
    G = O.G_tau(model, s, lt)
    S = [int(sw.X[b]), int(sw.Y[b])]
    sold = int(s[b, lt - 1])
    Δs = model.η[sx - 1] - model.η[sold - 1]
    t2 = np.array([Δs, model.a * Δs])
    t2 = np.exp(1j * t2) - 1 if model.is_complex else np.exp(t2) - 1
    r = np.eye(2) + t2[:, None] * (np.eye(2) - G[np.ix_(S, S)])
    d = np.linalg.det(r)
    p = abs(d) ** 2 if model.is_complex else float(np.real(d)) ** 2
    p *= model.γ[sx - 1] / model.γ[sold - 1]
    if not model.is_complex:
        p *= np.exp((model.η[sold - 1] - model.η[sx - 1]) * (model.a + 1))
    return p


@pytest.mark.parametrize("make,ratio", [(cases.tu_square, _ratio_tu), (cases.tu_honeycomb, _ratio_tu),
                                        (cases.tuv_honeycomb, _ratio_tuv),
                                        (lambda: cases.tuv_honeycomb(U=-4.0), _ratio_tuv)])
def test_log_weight_differences_are_the_acceptance_ratios(make, ratio):
    model = make()
    s = Initial_s(model, 9)
    rng = np.random.default_rng(4)
    w0 = log_weight(model, s, O.log_det(model, s)[0])
    assert abs(w0 - O.log_weight(model, s)) < 1e-9 * max(1.0, abs(w0))
    for _ in range(4):
        lt = int(rng.integers(1, model.Nt + 1))
        i = int(rng.integers(0, s.shape[0]))
        sx = int(rng.choice([v for v in (1, 2, 3, 4) if v != s[i, lt - 1]]))
        p = ratio(model, s, lt, i, sx)
        s2 = s.copy()
        s2[i, lt - 1] = sx
        w1 = log_weight(model, s2, O.log_det(model, s2)[0])
        assert abs((w1 - w0) - np.log(p)) < 1e-8, (w1 - w0, np.log(p))
