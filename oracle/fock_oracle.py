"""Exact many-body expectation values of the t-U projector sweep, summed in Fock space.

TEST INFRASTRUCTURE ONLY: a known-answer check for the Monte Carlo.  No
part of the product imports it.

The t-U sweep samples HS fields s with weight prod(gamma) |det(P^H B P)|^2,
B = B_Nt ... B_1, B_l = D_l eK, D_l = diag(cis(alpha_l eta_{s_il}))
(src/tU/GreenMatrix.jl:10-27, src/tU/phy_update.jl:259-261).  Written as
two fermion species a and b with ns = Ns/2 particles each, |det|^2 is the
overlap <Psi| T_Nt ... T_1 |Psi> of

    |Psi> = |P>_a (x) |conj P>_b,   T_l = V_l (Gamma(eK) (x) Gamma(conj eK)),
    V_l   = prod_i f_l(n_ai - n_bi),  f_l(m) = sum_k gamma_k exp(i alpha_l eta_k m),

where Gamma(M) is the Fock-space image of the one-particle matrix M (its
ns x ns minors) and the field sum has been done exactly, site by site.  A
measurement at tau = Nt/2 (the sweep wraps G there and conjugates it with
HalfeK, src/tU/phy_update.jl:154-190) is then the mixed expectation

    <O> = <Psi| T_Nt..T_{h+1} A^-1 O A T_h..T_1 |Psi> / <Psi| T_Nt..T_1 |Psi>,
    A = Gamma(HalfeK) (x) Gamma(conj HalfeK),  h = Nt/2,

with no Trotter, HS or projection approximation beyond the ones the
sweep itself makes: the Monte Carlo average of the sweep's per-sample
estimates must converge to it.  Feasible for Ns <= 12 (C(12,6)^2 states).
"""
from __future__ import annotations

from itertools import combinations

import numpy as np


def _basis(Ns: int, n: int):
    """Occupation sets of n particles on Ns sites, as sorted site tuples."""
    return list(combinations(range(Ns), n))


def gamma_op(M: np.ndarray, basis) -> np.ndarray:
    """Fock image of the one-particle matrix M: <S|Gamma(M)|T> = det M[S, T]."""
    idx = np.array(basis)
    sub = M[idx[:, None, :, None], idx[None, :, None, :]]
    return np.linalg.det(sub)


def slater(P: np.ndarray, basis) -> np.ndarray:
    """Amplitudes <S|P> = det P[S, :] of the Slater determinant of P's columns."""
    idx = np.array(basis)
    return np.linalg.det(P[idx, :])


def hop_op(i: int, j: int, basis) -> np.ndarray:
    """c_i^dagger c_j on the fixed-particle-number basis (sites ordered 0..Ns-1)."""
    pos = {S: k for k, S in enumerate(basis)}
    out = np.zeros((len(basis), len(basis)))
    for k, S in enumerate(basis):
        if j not in S:
            continue
        occ = list(S)
        sgn = (-1) ** occ.index(j)
        occ.remove(j)
        if i in occ:
            continue
        occ.append(i)
        occ.sort()
        sgn *= (-1) ** occ.index(i)
        out[pos[tuple(occ)], k] = sgn
    return out


def tu_exact(model):
    """Exact <Ek> and <Eu> of the t-U sweep's measurement at tau = Nt/2.

    Ek = -2 Ht Re sum_ij K_ij <c_ai c_aj^dagger> and Eu = Re sum_i <n_ai (1 - n_bi)>,
    the expectations of the sweep's per-sample estimates
    -2 Ht Re sum K .* G0 and sum_i (1 - G0_ii) conj(G0_ii)
    (src/tU/phy_update.jl:184-190).
    """
    Ns, Nt = model.Ns, model.Nt
    if Ns > 12:
        raise ValueError(f"Fock-space sum needs Ns <= 12, got {Ns}")
    ns = Ns // 2
    basis = _basis(Ns, ns)
    occ = np.zeros((len(basis), Ns))
    for k, S in enumerate(basis):
        occ[k, list(S)] = 1.0
    Ea, Eb = gamma_op(model.eK, basis), gamma_op(model.eK.conj(), basis)
    Ha, Hb = gamma_op(model.HalfeK, basis), gamma_op(model.HalfeK.conj(), basis)
    Hia, Hib = gamma_op(model.HalfeKinv, basis), gamma_op(model.HalfeKinv.conj(), basis)
    psi = np.outer(slater(model.Pt, basis), slater(model.Pt.conj(), basis))
    m = occ[:, None, :] - occ[None, :, :]                # n_a - n_b per site, (Sa, Sb, Ns)
    γ, η = np.asarray(model.γ), np.asarray(model.η)

    def V(l):  # slice l = 1..Nt
        f = {d: np.sum(γ * np.exp(1j * model.α[l - 1] * η * d)) for d in (-1, 0, 1)}
        return np.prod(np.select([m == -1, m == 0, m == 1], [f[-1], f[0], f[1]]), axis=2)

    h = Nt // 2
    R = psi.astype(np.complex128)
    for l in range(1, h + 1):
        R = V(l) * (Ea @ R @ Eb.T)
    L = psi.astype(np.complex128)
    for l in range(Nt, h, -1):          # T^H X = Ea^H (conj(V) * X) conj(Eb)
        L = Ea.conj().T @ (V(l).conj() * L) @ Eb.conj()
    norm = np.vdot(L, R)
    R1 = Ha @ R @ Hb.T                  # A |R>
    L1 = Hia.conj().T @ L @ Hib.conj()  # (A^-1)^H |L>

    def expect(X):
        return np.vdot(L1, X) / norm

    K = model.K
    Ek = 0.0 + 0.0j
    for i in range(Ns):
        for j in range(Ns):
            if K[i, j] == 0 and i != j:
                continue
            # <c_i c_j^dagger> = delta_ij - <c_j^dagger c_i>
            g = (1.0 if i == j else 0.0) - expect(hop_op(j, i, basis) @ R1)
            Ek += K[i, j] * g
    Ek = -2 * model.Ht * Ek.real
    nb1 = 1.0 - occ                                       # 1 - n_b, per b state
    Eu = sum(expect((occ[:, i][:, None] * nb1[:, i][None, :]) * R1) for i in range(Ns))
    return float(Ek), float(np.real(Eu))
