"""The oracle's Monte Carlo against the exact Fock-space sum of the same
weights (a known-answer test that does not share the oracle's arithmetic).

oracle/fock_oracle.py sums the sweep's weights over every HS field exactly,
in the Fock space of an 8-site lattice (two species for t-U and t-UV,
one for t-V), and returns the expectation of the sweep's per-sample
energy estimators at tau = Nt/2.  The oracle's chains must reproduce it
within five standard errors (independent chains, so the error bar is the
spread of the chain means).
"""
import numpy as np
import pytest

import cases
import dqmc_oracle as O
import fock_oracle as F
import philox
from kapdqmc_gb300 import Initial_s, tU_Hubbard_Para, tV_Hubbard_Para


def test_free_limit_is_exact():
    model = cases.tu_hc8(U=0.0)
    Ek, Eu = F.tu_exact(model)
    E = np.linalg.eigvalsh(model.K.real)
    assert abs(Ek - 2 * E[: model.Ns // 2].sum()) < 1e-9
    assert abs(Eu - model.Ns / 4) < 1e-9        # <n_up n_dn> = 1/4 per site


def _chains(model, nch, sweeps, cols, scale=None):
    n = O.proposals_per_sweep(model)
    means = []
    for c in range(nch):
        ks, us = zip(*(philox.tape(21, c, w, n) for w in range(sweeps)))
        sw = O.phy_update(model, Initial_s(model, 500 + c), sweeps,
                          O.Tape(np.concatenate(ks), np.concatenate(us)), True)
        means.append(np.array(sw.obs_rows)[10:, cols].mean(0) / (np.array(scale) if scale else 1.0))
    means = np.array(means)
    return means.mean(0), means.std(0, ddof=1) / np.sqrt(len(means))


def test_oracle_chains_reproduce_exact_sum():
    model = cases.tu_hc8()
    Ek, Eu = F.tu_exact(model)
    mu, se = _chains(model, 10, 100, [0, 1])
    assert abs(mu[0] - Ek) < 5 * se[0], (mu, se, Ek)
    assert abs(mu[1] - Eu) < 5 * se[1], (mu, se, Eu)
    # the interaction must be visible: U = 4 is many error bars from U = 0
    Ek0, Eu0 = F.tu_exact(cases.tu_hc8(U=0.0))
    assert abs(Eu0 - Eu) > 10 * se[1]


def test_tv_free_limit_and_oracle_chains():
    """t-V: the free limit, then Ek, Ev and the density structure factors
    R0, R1 (src/tV/phy_update.jl:268-294) of the oracle's chains."""
    Ek0, Ev0 = F.tv_exact(cases.tv_hc8(V=0.0))
    m0 = cases.tv_hc8(V=0.0)
    assert abs(Ek0 - np.linalg.eigvalsh(-m0.Ht * m0.K)[: m0.Ns // 2].sum()) < 1e-6
    model = cases.tv_hc8()
    Ek, Ev = F.tv_exact(model)
    R0, R1 = F.tv_structure_factors(model)
    want = np.concatenate([[Ek, Ev], R0, R1])
    mu, se = _chains(model, 8, 60, list(range(10)))
    assert np.all(np.abs(mu - want) < 5 * se + 1e-12), (mu, se, want)
    assert abs(Ev0 - Ev) > 10 * se[1]


@pytest.mark.parametrize("make", [cases.tuv_hc8, cases.tuv_hc8_real])
def test_tuv_oracle_chains(make):
    model = make()
    Ek, Eu = F.tuv_exact(model)
    mu, se = _chains(model, 6, 50, [0, 1], scale=(1.0, model.U))
    assert abs(mu[0] - Ek) < 5 * se[0], (mu, se, Ek)
    assert abs(mu[1] - Eu) < 5 * se[1], (mu, se, Eu)


def test_trotterised_projection_converges_to_hubbard_ground_state():
    """The exact sum of the sweep's weights (no sampling) against exact
    diagonalisation of the Hubbard Hamiltonian the model encodes: the total
    energy Ek + U Eu - U Ns/4 approaches E0 as dt shrinks (8-site honeycomb,
    U = 4, Theta = 3), which checks the model's K, alpha, gamma, eta and the
    sign conventions of the estimators against the physics."""
    U = 4.0

    def model(dt):
        return tU_Hubbard_Para(Ht=1.0, Hu1=U, Hu2=U, Δt=dt, Θrelax=3.0, Θquench=0.0,
                               Lattice="HoneyComb120", site=[2, 2], BatchSize=5, Initial="H0")

    E0, docc = F.hubbard_ground_state(model(0.1), U)
    errs = []
    for dt in (0.1, 0.05):
        m = model(dt)
        Ek, Eu = F.tu_exact(m)
        errs.append(abs(Ek + U * Eu - U * m.Ns / 4 - E0))
    assert errs[0] < 2e-3 and errs[1] < 2e-4 and errs[1] < errs[0] / 4, (E0, errs)
    Ek, Eu = F.tu_exact(model(0.05))
    assert abs(Eu - docc) < 1e-2, (Eu, docc)


def test_tv_trotterised_projection_converges_to_ground_state():
    """t-V: Ek + V (Ev - z Ns / 8) of the exact weight sum approaches the
    exact-diagonalisation ground state of the spinless t-V Hamiltonian."""
    V = 1.0

    def model(dt):
        return tV_Hubbard_Para(Ht=1.0, Hv1=V, Hv2=V, Δt=dt, Θrelax=3.0, Θquench=0.0,
                               Lattice="HoneyComb120", site=[2, 2], BatchSize=5, Initial="H0")

    m = model(0.1)
    E0, nxny = F.tv_ground_state(m, V)
    z = m.nnidx.shape[1]
    errs = []
    for dt in (0.1, 0.05):
        Ek, Ev = F.tv_exact(model(dt))
        errs.append(abs(Ek + V * (Ev - z * m.Ns / 8) - E0))
    assert errs[0] < 1e-4 and errs[1] < 1e-5 and errs[1] < errs[0] / 4, (E0, errs)
    assert abs(Ev - nxny) < 1e-2


def test_replica_estimator_identity_and_free_limit():
    """Rényi-2: for two field configurations, the Fock-space Tr(rho1_A rho2_A)
    of their two-species states at tau = Nt/2 equals the replica estimator
    |det(2 G1 G2 - G1 - G2 + I)_A|^2 on the restricted Green's functions (for
    regions that are not prefixes of the site order too); summed over the
    fields it is exact e^{-S2}, which at U = 0 is the free-fermion value."""
    m = cases.tu_hc8()
    s1, s2 = Initial_s(m, 1), Initial_s(m, 2)
    R1, L1, basis = F.tu_config_states(m, s1)
    R2, L2, _ = F.tu_config_states(m, s2)
    h = m.Nt // 2
    G1, G2 = O.G_tau(m, s1, h), O.G_tau(m, s2, h)
    for A in ([0, 1, 2, 3], [0, 2, 5], [1, 4, 6, 7], [3]):
        a, b = G1[np.ix_(A, A)], G2[np.ix_(A, A)]
        d = np.linalg.det(2 * a @ b - a - b + np.eye(len(A)))
        fock = F.tr_rho_rho(R1, L1, R2, L2, basis, A)
        assert abs(fock - abs(d) ** 2) < 1e-9 * max(1.0, abs(d) ** 2), (A, fock, abs(d) ** 2)
    m0 = cases.tu_hc8(U=0.0)
    A = [0, 1, 2, 3]
    G = np.eye(m0.Ns) - m0.Pt @ np.linalg.inv(m0.Pt.conj().T @ m0.Pt) @ m0.Pt.conj().T
    g = G[np.ix_(A, A)]
    free = abs(np.linalg.det(g @ g + (np.eye(4) - g) @ (np.eye(4) - g))) ** 2
    assert abs(F.tu_renyi2(m0, A) - free) < 1e-9
    assert 0.0 < F.tu_renyi2(m, A).real < 1.0


def test_scee_estimator_converges_to_exact_replica_ratio():
    """The coupled SCEE sweep (ctrl_SCEEicr restated) with lambda = 0 and
    N_lambda = 1 samples pairs with weight w(s1) w(s2) |det g_B|^2 and averages
    |det g_A|^2 / |det g_B|^2, so its estimator converges to
    Tr(rho_A^2) / Tr(rho_B^2) of the exact replica sums."""
    import scee_oracle as S
    m = cases.tu_hc8()
    A, B = [0, 1, 2, 3], [0, 1]
    exact = F.tu_renyi2(m, A).real / F.tu_renyi2(m, B).real
    n_rep = 2 * m.Ns * m.Nt
    means = []
    for p in range(5):
        sweeps = 100
        ks, us = [], []
        for w in range(sweeps):
            k0, u0 = philox.tape(5, 2 * p, w, n_rep)
            k1, u1 = philox.tape(5, 2 * p + 1, w, n_rep)
            ks.append(np.stack([k0, k1], axis=1).ravel())
            us.append(np.stack([u0, u1], axis=1).ravel())
        ref = S.SCEE(m, Initial_s(m, 300 + 2 * p), Initial_s(m, 301 + 2 * p), [a + 1 for a in A],
                     [b + 1 for b in B], 0.0, 1, O.Tape(np.concatenate(ks), np.concatenate(us))).run(sweeps)
        means.append(np.mean(ref.O[20:]))
    mu, se = np.mean(means), np.std(means, ddof=1) / np.sqrt(len(means))
    assert abs(mu - exact) < 5 * se, (mu, se, exact)
    assert se < 0.1 * exact


def test_dop_estimator_converges_to_exact_disorder_ratio():
    """ctrl_SCDOPicr restated, lambda = 0, N_lambda = 1: the chain is weighted by
    |det X_B|^2 and averages |det X_A|^2 / |det X_B|^2, whose exact value is
    <exp(i alpha (N_a,A - N_b,A))> / <... B ...> in the sweep's two-species
    state (fock_oracle.tu_disorder); at U = 0 the exact sum is the Slater
    value |det X_A|^2."""
    import scee_oracle as S
    m = cases.tu_hc8()
    A, B, alpha = [0, 1, 2, 3], [0, 1], 1.0
    m0 = cases.tu_hc8(U=0.0)
    G = np.eye(m0.Ns) - m0.Pt @ np.linalg.inv(m0.Pt.conj().T @ m0.Pt) @ m0.Pt.conj().T
    e = np.exp(1j * alpha)
    X = e * np.eye(4) + (1 - e) * G[np.ix_(A, A)]
    assert abs(F.tu_disorder(m0, A, alpha) - abs(np.linalg.det(X)) ** 2) < 1e-9
    exact = (F.tu_disorder(m, A, alpha) / F.tu_disorder(m, B, alpha)).real
    means = []
    for c in range(8):
        sweeps = 120
        ks, us = zip(*(philox.tape(8, c, w, 2 * m.Ns * m.Nt) for w in range(sweeps)))
        ref = S.DOP(m, Initial_s(m, 400 + c), alpha, [a + 1 for a in A], [b + 1 for b in B], 0.0, 1,
                    O.Tape(np.concatenate(ks), np.concatenate(us))).run(sweeps)
        means.append(np.mean(ref.O[20:]))
    mu, se = np.mean(means), np.std(means, ddof=1) / np.sqrt(len(means))
    assert abs(mu - exact) < 5 * se, (mu, se, exact)
    assert se < 0.02


def test_full_structure_factors_converge_to_exact_correlations():
    """The structure factors with every term (kdq_set_measure_full; the
    oracle's full_sf) average to the staggered charge and spin correlations
    of the exact state: CDW = sum_{c1,c2} w <(rho_A1 - rho_B1)(rho_A2 - rho_B2)> / Ns^2
    with rho = n_up + n_dn (SDW with n_up - n_dn)."""
    m = cases.tu_hc8()
    exact = np.array(F.tu_structure_factors(m))
    n = O.proposals_per_sweep(m)
    means = []
    for c in range(12):
        sweeps = 150
        ks, us = zip(*(philox.tape(77, c, w, n) for w in range(sweeps)))
        sw = O.phy_update(m, Initial_s(m, 700 + c), sweeps, O.Tape(np.concatenate(ks), np.concatenate(us)),
                          True, full_sf=True)
        means.append(np.array(sw.obs_rows)[20:, 6:10].mean(0))
    means = np.array(means)
    mu, se = means.mean(0), means.std(0, ddof=1) / np.sqrt(len(means))
    assert np.all(np.abs(mu - exact) < 5 * se), (mu, se, exact)
    assert np.all(se < 0.1 * np.abs(exact))


def test_square_staggered_structure_factors_converge_to_exact_correlations():
    """On a square lattice the full-measurement columns 6 and 8 are the
    staggered charge and spin structure factors at (pi, pi) (no counterpart
    in the reference, whose square branch measures none): the oracle's
    chains average to the exact sum_ij e_i e_j <rho_i rho_j> / Ns^2 of the
    8-site torus."""
    m = cases.tu_sq8()
    exact = np.array(F.tu_staggered_structure_factors(m))
    n = O.proposals_per_sweep(m)
    means = []
    for c in range(12):
        sweeps = 150
        ks, us = zip(*(philox.tape(78, c, w, n) for w in range(sweeps)))
        sw = O.phy_update(m, Initial_s(m, 710 + c), sweeps, O.Tape(np.concatenate(ks), np.concatenate(us)),
                          True, full_sf=True)
        rows = np.array(sw.obs_rows)
        assert np.all(rows[:, 7] == 0) and np.all(rows[:, 9] == 0)
        means.append(rows[20:, [6, 8]].mean(0))
    means = np.array(means)
    mu, se = means.mean(0), means.std(0, ddof=1) / np.sqrt(len(means))
    assert np.all(np.abs(mu - exact) < 5 * se), (mu, se, exact)
    assert np.all(se < 0.1 * np.abs(exact))
