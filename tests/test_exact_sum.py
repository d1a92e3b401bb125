"""The oracle's Monte Carlo against the exact Fock-space sum of the same
weights (a known-answer test that does not share the oracle's arithmetic).

oracle/fock_oracle.py sums the t-U sweep's weights over every HS field
exactly, in the two-species Fock space of an 8-site lattice, and returns the
expectation of the sweep's per-sample energy estimators at tau = Nt/2.  The
oracle's chains must reproduce it within five standard errors (independent
chains, so the error bar is the spread of the chain means).
"""
import numpy as np

import cases
import dqmc_oracle as O
import fock_oracle as F
import philox
from kapdqmc_gb300 import Initial_s


def test_free_limit_is_exact():
    model = cases.tu_hc8(U=0.0)
    Ek, Eu = F.tu_exact(model)
    E = np.linalg.eigvalsh(model.K.real)
    assert abs(Ek - 2 * E[: model.Ns // 2].sum()) < 1e-9
    assert abs(Eu - model.Ns / 4) < 1e-9        # <n_up n_dn> = 1/4 per site


def test_oracle_chains_reproduce_exact_sum():
    model = cases.tu_hc8()
    Ek, Eu = F.tu_exact(model)
    n = O.proposals_per_sweep(model)
    means = []
    for c in range(10):
        sweeps = 100
        ks, us = zip(*(philox.tape(21, c, w, n) for w in range(sweeps)))
        sw = O.phy_update(model, Initial_s(model, 500 + c), sweeps,
                          O.Tape(np.concatenate(ks), np.concatenate(us)), True)
        means.append(np.array(sw.obs_rows)[10:, :2].mean(0))
    means = np.array(means)
    mu, se = means.mean(0), means.std(0, ddof=1) / np.sqrt(len(means))
    assert abs(mu[0] - Ek) < 5 * se[0], (mu, se, Ek)
    assert abs(mu[1] - Eu) < 5 * se[1], (mu, se, Eu)
    # the interaction must be visible: U = 4 is many error bars from U = 0
    Ek0, Eu0 = F.tu_exact(cases.tu_hc8(U=0.0))
    assert abs(Eu0 - Eu) > 10 * se[1]
