"""Cluster moves of the oracle's t-U sweep (CPU): G stays the brute-force
Green's function of the updated fields, and the exact multi-site ratio
|det(I + Delta_S (I - G_SS))|^2 prod gamma'/gamma equals the change of the
log-weight."""
import numpy as np
import pytest

import cases
import cnn_oracle as N
import dqmc_oracle as O
import philox
from kapdqmc_gb300 import Initial_s
from kapdqmc_gb300.sweep import log_weight


@pytest.mark.parametrize("zero", [True, False])
def test_cluster_moves_keep_G_consistent(zero):
    m = cases.tu_square()
    s0 = Initial_s(m, 3)
    n = O.proposals_per_sweep(m)
    ks, us = zip(*(philox.tape(5, 0, w, n) for w in range(2)))
    params = np.zeros(N.NPARAM, np.float32) if zero else N.init_params(2) * 0.3
    cfg = dict(params=params, moves=1, cluster_len=4, steps=8, seed=5, chain=0)
    r = O.phy_update(m, s0, 2, O.Tape(np.concatenate(ks), np.concatenate(us)), False, slmc=cfg)
    Gt = O.G_tau(m, r.s, 0)
    assert np.linalg.norm(r.G - Gt) / np.linalg.norm(Gt) < 1e-10
    assert max(r.drift) < 1e-8
    final = [p for p in r.slmc_log]
    assert len(final) >= 2 * 2 * m.Nt * 8    # every effective step is logged
    assert not np.array_equal(r.s, s0)


def test_multi_site_ratio_is_the_weight_change():
    m = cases.tu_honeycomb()
    s = Initial_s(m, 8)
    rng = np.random.default_rng(1)
    for _ in range(3):
        lt = int(rng.integers(1, m.Nt + 1))
        idx = sorted(rng.choice(m.Ns, 5, replace=False).tolist())
        new = [int(rng.choice([v for v in (1, 2, 3, 4) if v != s[i, lt - 1]])) for i in idx]
        G = O.G_tau(m, s, lt)
        old = [int(s[i, lt - 1]) for i in idx]
        Δ = np.array([np.exp(1j * m.α[lt - 1] * (m.η[b - 1] - m.η[a - 1])) - 1 for a, b in zip(old, new)])
        M = np.eye(len(idx)) + Δ[:, None] * (np.eye(len(idx)) - G[np.ix_(idx, idx)])
        lr = 2 * np.log(abs(np.linalg.det(M))) + sum(np.log(m.γ[b - 1] / m.γ[a - 1]) for a, b in zip(old, new))
        s2 = s.copy()
        for i, v in zip(idx, new):
            s2[i, lt - 1] = v
        dw = log_weight(m, s2, O.log_det(m, s2)[0]) - log_weight(m, s, O.log_det(m, s)[0])
        assert abs(dw - lr) < 1e-8, (dw, lr)
