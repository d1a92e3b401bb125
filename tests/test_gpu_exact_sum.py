"""The CUDA sweep's observables against the exact Fock-space sum of its weights.

oracle/fock_oracle.py sums the weights of the t-U, t-V and complex t-UV
sweeps over every HS field exactly on 8- and 12-site lattices and returns
the expectation of the sweep's two energy estimators (columns 0 and 1) at
tau = Nt/2.  Hundreds of independent GPU chains must reproduce it within
five standard errors: in FP64, in mixed precision, with a slice-dependent
coupling (quench), with a complex hopping matrix (pi flux) and with the
self-learning cluster moves switched on (their exact acceptance must leave
the distribution unchanged whatever the network proposes).
"""
import numpy as np
import pytest

import cases
import fock_oracle as F
from kapdqmc_gb300 import Initial_s, slmc
from kapdqmc_gb300.model import KIND_TU, KIND_TUV, KIND_TV
from kapdqmc_gb300.sweep import Sweeper

pytestmark = pytest.mark.gpu

WARM, SWEEPS = 20, 220


def _run(model, nchains, precision="fp64", seed=4321, slmc_args=None):
    fields = np.stack([Initial_s(model, 9000 + c) for c in range(nchains)])
    with Sweeper(model, nchains) as sw:
        sw.set_precision(precision)
        if slmc_args is not None:
            sw.slmc_enable(*slmc_args)
        sw.set_fields(fields)
        sw.set_rng(seed)
        obs = sw.phy_update(SWEEPS, True)
        st = sw.slmc_stats() if slmc_args is not None else None
    chain_means = obs[:, WARM:, :2].mean(axis=1)
    mu = chain_means.mean(axis=0)
    se = chain_means.std(axis=0, ddof=1) / np.sqrt(nchains)
    return mu, se, st


def _exact(model):
    if model.kind == KIND_TU:
        return F.tu_exact(model)
    if model.kind == KIND_TV:
        return F.tv_exact(model)
    Ek, Eu = F.tuv_exact(model)
    return Ek, model.U * Eu          # column 1 of t-UV is U * Eu


def _check(model, mu, se):
    Ek, Eu = _exact(model)
    assert abs(mu[0] - Ek) < 5 * se[0] + 1e-9, (mu[0], se[0], Ek)
    assert abs(mu[1] - Eu) < 5 * se[1] + 1e-9, (mu[1], se[1], Eu)
    # the run resolves the answer (the pi-flux lattice's Ek estimator averages to 0)
    assert se[0] < 0.02 * max(1.0, abs(Ek))


@pytest.mark.parametrize("make", [cases.tu_hc8, cases.tu_hc8_quench, cases.tu_sq8, cases.tu_sq8_flux,
                                  cases.tuv_hc8])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_sweep_reproduces_exact_sum(make, precision):
    model = make()
    mu, se, _ = _run(model, 512, precision)
    _check(model, mu, se)


def test_tv_sweep_reproduces_exact_sum():
    model = cases.tv_hc8()             # real HS factors: FP64 only
    mu, se, _ = _run(model, 512, "fp64")
    _check(model, mu, se)


def test_cluster_moves_keep_the_distribution():
    model = cases.tu_hc12()
    params = (slmc.init_params(5) * 0.05).astype(np.float32)
    mu, se, st = _run(model, 256, "fp64", slmc_args=(params, 1, 4, 16))
    assert st["proposed"] > 0 and 0 < st["accepted"] < st["proposed"]
    _check(model, mu, se)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_square_staggered_structure_factors_reproduce_exact_sum(precision):
    """Full-measurement columns 6 and 8 on the 8-site square torus: the
    staggered charge and spin structure factors at (pi, pi)."""
    model = cases.tu_sq8()
    exact = np.array(F.tu_staggered_structure_factors(model))
    fields = np.stack([Initial_s(model, 9100 + c) for c in range(512)])
    with Sweeper(model, 512) as sw:
        sw.set_precision(precision)
        sw.set_measure_full(True)
        sw.set_fields(fields)
        sw.set_rng(2468)
        obs = sw.phy_update(SWEEPS, True)
    chain_means = obs[:, WARM:, [6, 8]].mean(axis=1)
    mu = chain_means.mean(axis=0)
    se = chain_means.std(axis=0, ddof=1) / np.sqrt(len(chain_means))
    assert np.all(np.abs(mu - exact) < 5 * se), (mu, se, exact)
    assert np.all(se < 0.05 * np.abs(exact))
