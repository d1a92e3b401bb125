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
import scipy.linalg


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


def _two_species(model, V, ek_sign, same_species=False):
    """<Ek>, <Eu> of a two-species sweep: V(l) is the diagonal field-summed
    interaction of slice l over (a state, b state).  Eu is
    sum_i <n_ai (1 - n_bi)> for |det|^2 weights (species b the conjugate of a,
    whose per-sample estimator is (1 - G_ii) conj(G_ii)) or, with
    same_species, sum_i <n_ai n_bi> for det^2 weights (estimator (1 - G_ii)^2)."""
    Ns, Nt = model.Ns, model.Nt
    if Ns > 12:
        raise ValueError(f"Fock-space sum needs Ns <= 12, got {Ns}")
    basis = _basis(Ns, Ns // 2)
    occ = _occupations(basis, Ns)
    Ea, Eb = gamma_op(model.eK, basis), gamma_op(model.eK.conj(), basis)
    Ha, Hb = gamma_op(model.HalfeK, basis), gamma_op(model.HalfeK.conj(), basis)
    Hia, Hib = gamma_op(model.HalfeKinv, basis), gamma_op(model.HalfeKinv.conj(), basis)
    psi = np.outer(slater(model.Pt, basis), slater(model.Pt.conj(), basis)).astype(np.complex128)
    h = Nt // 2
    R = psi.copy()
    for l in range(1, h + 1):           # rescaled every slice: <O> is a ratio
        R = V(l) * (Ea @ R @ Eb.T)
        R /= np.linalg.norm(R)
    L = psi.copy()
    for l in range(Nt, h, -1):          # T^H X = Ea^H (conj(V) * X) conj(Eb)
        L = Ea.conj().T @ (V(l).conj() * L) @ Eb.conj()
        L /= np.linalg.norm(L)
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
    Ek = ek_sign * 2 * model.Ht * Ek.real
    nb = occ if same_species else 1.0 - occ               # n_b or 1 - n_b, per b state
    Eu = sum(expect((occ[:, i][:, None] * nb[:, i][None, :]) * R1) for i in range(Ns))
    return float(Ek), float(np.real(Eu))


def _occupations(basis, Ns):
    occ = np.zeros((len(basis), Ns))
    for k, S in enumerate(basis):
        occ[k, list(S)] = 1.0
    return occ


def tu_exact(model):
    """Exact <Ek> and <Eu> of the t-U sweep's measurement at tau = Nt/2.

    Ek = -2 Ht Re sum_ij K_ij <c_ai c_aj^dagger> and Eu = Re sum_i <n_ai (1 - n_bi)>,
    the expectations of the sweep's per-sample estimates
    -2 Ht Re sum K .* G0 and sum_i (1 - G0_ii) conj(G0_ii)
    (src/tU/phy_update.jl:184-190).
    """
    occ = _occupations(_basis(model.Ns, model.Ns // 2), model.Ns)
    m = occ[:, None, :] - occ[None, :, :]                # n_a - n_b per site, (Sa, Sb, Ns)
    γ, η = np.asarray(model.γ), np.asarray(model.η)

    def V(l):  # slice l = 1..Nt
        f = {d: np.sum(γ * np.exp(1j * model.α[l - 1] * η * d)) for d in (-1, 0, 1)}
        return np.prod(np.select([m == -1, m == 0, m == 1], [f[-1], f[0], f[1]]), axis=2)

    return _two_species(model, V, -1.0)


def tuv_exact(model):
    """Exact <Ek> and <Eu> / U of the t-UV sweep at tau = Nt/2.

    One field per bond (x, y) and slice multiplies species a by
    exp(i eta (n_x + a n_y)) and species b by its conjugate
    (src/tUV/GreenMatrix.jl:10-36, src/tUV/phy_update.jl:188-203), so the
    field sum of a bond is f(m) = sum_k gamma_k exp(i eta_k m) with
    m = (n_ax + a n_ay) - (n_bx + a n_by).  Returns 2 Ht Re sum K .* G0 and
    Re sum_i <n_ai (1 - n_bi)> (the sweep's Ek and Eu / U,
    src/tUV/phy_update.jl:205-235).
    """
    occ = _occupations(_basis(model.Ns, model.Ns // 2), model.Ns)
    nn = np.asarray(model.nnidx)
    X = nn[:, :, 0].ravel(order="F") - 1
    Y = nn[:, :, 1].ravel(order="F") - 1
    γ, η = np.asarray(model.γ), np.asarray(model.η)
    qa = occ[:, X] + model.a * occ[:, Y]                  # per a state and bond
    if model.is_complex:
        m = qa[:, None, :] - qa[None, :, :]               # (Sa, Sb, bonds)
        f = np.tensordot(np.exp(1j * m[..., None] * η), γ, axes=([3], [0]))
    else:
        # real sweep: both species see exp(+eta (n_x + a n_y)) and each field
        # carries exp(-(a + 1) eta) (src/tUV/phy_update.jl:195-197), weight det^2
        m = qa[:, None, :] + qa[None, :, :]
        f = np.tensordot(np.exp(m[..., None] * η), γ * np.exp(-(model.a + 1.0) * η), axes=([3], [0]))
    Vc = np.prod(f, axis=2)                               # the same for every slice

    return _two_species(model, lambda l: Vc, 1.0, same_species=not model.is_complex)


def tv_states(model):
    """(R1, L1, basis): the t-V sweep's one-species states at tau = Nt/2 with
    the HalfeK symmetrisation of the measurement, R1 = A T_h .. T_1 |Psi>,
    L1 = (A^-1)^H T_{h+1}^H .. T_Nt^H |Psi>, A = Gamma(HalfeK).  A bond (x, y)
    of direction j acts on its two sites by UV diag(exp(alpha eta),
    exp(-alpha eta)) UV, UV = [-c -c; -c c], c = 1/sqrt 2, and its field sum is
    sum_k gamma_k Gamma(that matrix); B_l = prod_j (UV_j D_j UV_j) eK
    (src/tV/GreenMatrix.jl:12-38)."""
    Ns, Nt = model.Ns, model.Nt
    if Ns > 12:
        raise ValueError(f"Fock-space sum needs Ns <= 12, got {Ns}")
    basis = _basis(Ns, Ns // 2)
    nn = np.asarray(model.nnidx)
    γ, η = np.asarray(model.γ), np.asarray(model.η)
    c = 2 ** 0.5 / 2
    UV = np.array([[-c, -c], [-c, c]])

    def V(l):
        out = np.eye(len(basis))
        for j in range(nn.shape[1]):                  # B = (UV_1 D_1 UV_1)(UV_2 D_2 UV_2)... eK
            Vj = np.eye(len(basis))
            for b in range(nn.shape[0]):
                x, y = nn[b, j] - 1
                S = 0
                for g, e in zip(γ, η):
                    v = model.α[l - 1] * e
                    M = np.eye(Ns)
                    M[np.ix_([x, y], [x, y])] = UV @ np.diag([np.exp(v), np.exp(-v)]) @ UV
                    S = S + g * gamma_op(M, basis)
                Vj = Vj @ S
            out = out @ Vj
        return out

    E = gamma_op(model.eK, basis)
    H, Hi = gamma_op(model.HalfeK, basis), gamma_op(model.HalfeKinv, basis)
    psi = slater(model.Pt, basis)
    h = Nt // 2
    Vs = {}

    def Vl(l):
        key = float(model.α[l - 1])
        if key not in Vs:
            Vs[key] = V(l)
        return Vs[key]

    R = psi.copy()
    for l in range(1, h + 1):           # rescaled every slice: <O> is a ratio
        R = Vl(l) @ (E @ R)
        R /= np.linalg.norm(R)
    L = psi.copy()
    for l in range(Nt, h, -1):
        L = E.conj().T @ (Vl(l).conj().T @ L)
        L /= np.linalg.norm(L)
    return H @ R, Hi.conj().T @ L, basis


def tv_exact(model):
    """Exact <Ek> and <Ev> of the t-V sweep's measurement at tau = Nt/2: one
    fermion species with weight prod(gamma) det(P^H B P) (see tv_states).
    Returns Ht sum K .* <c c^dagger> and sum_bonds <n_x n_y>, the
    expectations of the sweep's Ek and Ev (src/tV/phy_update.jl:207-262)."""
    Ns = model.Ns
    R1, L1, basis = tv_states(model)
    occ = _occupations(basis, Ns)
    norm = np.vdot(L1, R1)

    def expect(v):
        return np.vdot(L1, v) / norm

    K = model.K
    Ek = 0.0
    for i in range(Ns):
        for j in range(Ns):
            if K[i, j] == 0 and i != j:
                continue
            g = (1.0 if i == j else 0.0) - expect(hop_op(j, i, basis) @ R1)
            Ek += K[i, j] * g
    nn = np.asarray(model.nnidx)
    x = nn[:, :, 0].ravel() - 1
    y = nn[:, :, 1].ravel() - 1
    Ev = expect((occ[:, x] * occ[:, y]).sum(axis=1) * R1)
    return float(np.real(model.Ht * Ek)), float(np.real(Ev))


def tv_structure_factors(model):
    """Exact R0[4], R1[4] of the t-V honeycomb measurement: for cells c1, c2
    and the sublattice pairs (A,A), (B,B), (B1,A2), (A1,B2),
    4 / Ns^2 sum_{c1,c2} w <n_X1 n_Y2> with w = 1 (R0) or
    cos(2 pi rx / L1 + 2 pi ry / L2) (R1) (src/tV/phy_update.jl:268-294)."""
    R1, L1, basis = tv_states(model)
    occ = _occupations(basis, model.Ns)
    norm = np.vdot(L1, R1)
    L1_, L2_ = model.site
    cells = {(ix, iy): 2 * (ix + (iy - 1) * L1_) - 2 for ix in range(1, L1_ + 1) for iy in range(1, L2_ + 1)}
    R0, Rq = np.zeros(4), np.zeros(4)
    for (ix, iy), a1 in cells.items():
        for rx in range(1, L1_ + 1):
            for ry in range(1, L2_ + 1):
                a2 = cells[((ix + rx - 1) % L1_ + 1, (iy + ry - 1) % L2_ + 1)]
                b1, b2 = a1 + 1, a2 + 1
                ph = np.cos(2 * np.pi / L1_ * rx + 2 * np.pi / L2_ * ry)
                for k, (p, q) in enumerate(((a1, a2), (b1, b2), (b1, a2), (a1, b2))):
                    v = np.real(np.vdot(L1, occ[:, p] * occ[:, q] * R1) / norm)
                    R0[k] += v
                    Rq[k] += ph * v
    return R0 * 4 / model.Ns ** 2, Rq * 4 / model.Ns ** 2


def hubbard_ground_state(model, U: float):
    """Ground-state energy and double occupancy sum_i <n_i,up n_i,dn> of
    H = Ht sum_s c_s^dagger K c_s + U sum_i (n_i,up - 1/2)(n_i,dn - 1/2) at half
    filling, by exact diagonalisation (dense, Ns <= 8): the Hamiltonian the
    t-U sweep's Trotterised projection converges to as dt -> 0, Theta -> oo
    (the model's Hu1 = Hu2 = U, src/tU/model.jl:39-96)."""
    Ns = model.Ns
    if Ns > 8:
        raise ValueError(f"dense diagonalisation needs Ns <= 8, got {Ns}")
    basis = _basis(Ns, Ns // 2)
    D = len(basis)
    occ = _occupations(basis, Ns)
    K = np.asarray(model.K)
    K = K.real if not np.any(np.imag(K)) else K
    Hk = np.zeros((D, D), dtype=K.dtype)
    for i in range(Ns):
        for j in range(Ns):
            if K[i, j] != 0:
                Hk += K[i, j] * hop_op(i, j, basis)
    eye = np.eye(D)
    H = model.Ht * (np.kron(Hk, eye) + np.kron(eye, Hk))
    pair = (occ[:, None, :] - 0.5) * (occ[None, :, :] - 0.5)       # (up state, dn state, site)
    H += np.diag(U * pair.sum(axis=2).reshape(D * D))
    w, v = scipy.linalg.eigh(H, subset_by_index=[0, 0])
    g = np.abs(v[:, 0]) ** 2
    docc = float(((occ[:, None, :] * occ[None, :, :]).sum(axis=2).reshape(D * D) * g).sum())
    return float(w[0]), docc


def tv_ground_state(model, V: float):
    """Ground-state energy and sum_bonds <n_x n_y> of the spinless
    H = -Ht c^dagger K c + V sum_bonds (n_x - 1/2)(n_y - 1/2) at half filling,
    by exact diagonalisation: the Hamiltonian the t-V sweep's Trotterised
    projection converges to (the model's Hv1 = Hv2 = V, src/tV/model.jl:30-122)."""
    Ns = model.Ns
    if Ns > 12:
        raise ValueError(f"dense diagonalisation needs Ns <= 12, got {Ns}")
    basis = _basis(Ns, Ns // 2)
    occ = _occupations(basis, Ns)
    K = np.asarray(model.K).real
    H = np.zeros((len(basis), len(basis)))
    for i in range(Ns):
        for j in range(Ns):
            if K[i, j] != 0:
                H -= model.Ht * K[i, j] * hop_op(i, j, basis)
    nn = np.asarray(model.nnidx)
    x, y = nn[:, :, 0].ravel() - 1, nn[:, :, 1].ravel() - 1
    H += np.diag(V * ((occ[:, x] - 0.5) * (occ[:, y] - 0.5)).sum(axis=1))
    w, v = np.linalg.eigh(H)
    return float(w[0]), float(((occ[:, x] * occ[:, y]).sum(axis=1) * v[:, 0] ** 2).sum())


def _split_sign(S, A):
    """Sign of reordering the occupied modes S (ascending sites) so that the
    sites in A come first (each in ascending order)."""
    inv, seen_b = 0, 0
    for i in S:
        if i in A:
            inv += seen_b
        else:
            seen_b += 1
    return -1.0 if inv & 1 else 1.0


def _region_split(basis, A):
    """Row (region) and column (rest) index and sign of every two-species
    basis state (Sa, Sb), modes reordered as (a_A, b_A, a_B, b_B)."""
    keyA, keyB = {}, {}
    rows, cols, sg = [], [], []
    for Sa in basis:
        aA = tuple(i for i in Sa if i in A)
        aB = tuple(i for i in Sa if i not in A)
        for Sb in basis:
            bA = tuple(i for i in Sb if i in A)
            bB = tuple(i for i in Sb if i not in A)
            s = _split_sign(Sa, A) * _split_sign(Sb, A) * (-1.0 if (len(bA) * len(aB)) & 1 else 1.0)
            rows.append(keyA.setdefault((aA, bA), len(keyA)))
            cols.append(keyB.setdefault((aB, bB), len(keyB)))
            sg.append(s)
    return np.array(rows), np.array(cols), np.array(sg), (len(keyA), len(keyB))


def tr_rho_rho(R1, L1, R2, L2, basis, A):
    """Tr(rho1_A rho2_A) for the two-species operators rho_k = |R_k><L_k| / <L_k|R_k>
    (R, L as (a state, b state) amplitude matrices), A a set of 0-based sites."""
    rows, cols, sg, shape = _region_split(basis, set(int(a) for a in A))

    def mat(X):
        P = np.zeros(shape, dtype=np.complex128)
        P[rows, cols] = sg * X.ravel()
        return P

    r1 = mat(R1) @ mat(L1).conj().T / np.vdot(L1, R1)
    r2 = mat(R2) @ mat(L2).conj().T / np.vdot(L2, R2)
    return complex(np.trace(r1 @ r2))


def tu_states(model, V):
    """R = T_h .. T_1 |Psi> and L = T_{h+1}^H .. T_Nt^H |Psi> (h = Nt/2) of the
    two-species t-U transfer matrices with slice interactions V(l)."""
    Ns, Nt = model.Ns, model.Nt
    basis = _basis(Ns, Ns // 2)
    Ea, Eb = gamma_op(model.eK, basis), gamma_op(model.eK.conj(), basis)
    psi = np.outer(slater(model.Pt, basis), slater(model.Pt.conj(), basis)).astype(np.complex128)
    h = Nt // 2
    R = psi.copy()
    for l in range(1, h + 1):
        R = V(l) * (Ea @ R @ Eb.T)
        R /= np.linalg.norm(R)
    L = psi.copy()
    for l in range(Nt, h, -1):
        L = Ea.conj().T @ (V(l).conj() * L) @ Eb.conj()
        L /= np.linalg.norm(L)
    return R, L, basis


def tu_config_states(model, s):
    """tu_states for one field configuration s (Ns x Nt): species a sees
    cis(alpha eta) on occupied sites, species b its conjugate."""
    basis = _basis(model.Ns, model.Ns // 2)
    occ = _occupations(basis, model.Ns)
    η = np.asarray(model.η)

    def V(l):
        ph = model.α[l - 1] * η[np.asarray(s)[:, l - 1].astype(np.int64) - 1]
        fa = np.exp(1j * occ @ ph)
        return np.outer(fa, fa.conj())

    return tu_states(model, V)


def tu_renyi2(model, A):
    """Exact e^{-S2} = Tr(rho_A^2) of the t-U sweep's two-species state at
    tau = Nt/2, rho = |R><L| / <L|R> with R = T_h .. T_1 |Psi>,
    <L| = <Psi| T_Nt .. T_{h+1} (the field sums of tu_exact), and A a set of
    0-based sites taken in both species.  This is what the replica estimator
    |det(2 G1 G2 - G1 - G2 + I)_A|^2 over independent pairs of the sweep's
    configurations at tau = Nt/2 converges to (GroverMatrix!,
    src/public/GF.jl:101-109; |det|^2 as in src/tU/SCEE.jl:264-276)."""
    if model.Ns > 8:
        raise ValueError(f"Fock-space replica sum needs Ns <= 8, got {model.Ns}")
    occ = _occupations(_basis(model.Ns, model.Ns // 2), model.Ns)
    m = occ[:, None, :] - occ[None, :, :]
    γ, η = np.asarray(model.γ), np.asarray(model.η)

    def V(l):
        f = {d: np.sum(γ * np.exp(1j * model.α[l - 1] * η * d)) for d in (-1, 0, 1)}
        return np.prod(np.select([m == -1, m == 0, m == 1], [f[-1], f[0], f[1]]), axis=2)

    R, L, basis = tu_states(model, V)
    return tr_rho_rho(R, L, R, L, basis, A)


def tu_disorder(model, region, alpha: float):
    """Exact <exp(i alpha (N_a,R - N_b,R))> of the t-U sweep's two-species state
    at tau = Nt/2 (region R: 0-based sites): the average over the sweep's
    configurations of |det X_R|^2, X = e^{i alpha} I + (1 - e^{i alpha}) G[R,R]
    (the disorder operator of ctrl_SCDOPicr, src/tU/disorder_operate.jl:202-224),
    since det X_R is the Slater expectation of exp(i alpha N_R) of species a and
    its conjugate that of exp(-i alpha N_R) of species b."""
    if model.Ns > 12:
        raise ValueError(f"Fock-space sum needs Ns <= 12, got {model.Ns}")
    occ = _occupations(_basis(model.Ns, model.Ns // 2), model.Ns)
    m = occ[:, None, :] - occ[None, :, :]
    γ, η = np.asarray(model.γ), np.asarray(model.η)

    def V(l):
        f = {d: np.sum(γ * np.exp(1j * model.α[l - 1] * η * d)) for d in (-1, 0, 1)}
        return np.prod(np.select([m == -1, m == 0, m == 1], [f[-1], f[0], f[1]]), axis=2)

    R, L, _ = tu_states(model, V)
    nR = occ[:, list(region)].sum(axis=1)
    D = np.exp(1j * alpha * (nR[:, None] - nR[None, :]))
    return complex(np.vdot(L, D * R) / np.vdot(L, R))


def tu_structure_factors(model):
    """Exact CDW0, CDW1, SDW0, SDW1 of the t-U honeycomb sweep's measurement
    with every term (the estimator kdq_set_measure_full adds): with
    n_up = n_a and n_dn = 1 - n_b (species b is the particle-hole conjugate of
    spin down), rho = n_up + n_dn and m = n_up - n_dn, and for cells c1, c2 with
    A and B sites, CDW = sum_{c1,c2} w(c2 - c1) <(rho_A1 - rho_B1)(rho_A2 - rho_B2)> / Ns^2
    (SDW with m), w = 1 (…0) or cos(2 pi rx / L1 + 2 pi ry / L2) (…1); the
    reference's correlators, src/tU/phy_update.jl:194-235, with their
    discarded +adjoint terms restored."""
    Ns = model.Ns
    if Ns > 12:
        raise ValueError(f"Fock-space sum needs Ns <= 12, got {Ns}")
    basis = _basis(Ns, Ns // 2)
    occ = _occupations(basis, Ns)
    m = occ[:, None, :] - occ[None, :, :]
    γ, η = np.asarray(model.γ), np.asarray(model.η)

    def V(l):
        f = {d: np.sum(γ * np.exp(1j * model.α[l - 1] * η * d)) for d in (-1, 0, 1)}
        return np.prod(np.select([m == -1, m == 0, m == 1], [f[-1], f[0], f[1]]), axis=2)

    R, L, _ = tu_states(model, V)
    Ha, Hb = gamma_op(model.HalfeK, basis), gamma_op(model.HalfeK.conj(), basis)
    Hia, Hib = gamma_op(model.HalfeKinv, basis), gamma_op(model.HalfeKinv.conj(), basis)
    R1 = Ha @ R @ Hb.T
    L1 = Hia.conj().T @ L @ Hib.conj()
    norm = np.vdot(L1, R1)
    nup = occ[:, None, :]                       # (Sa, 1, site)
    ndn = 1.0 - occ[None, :, :]                 # (1, Sb, site)
    L1_, L2_ = model.site
    cells = {(ix, iy): 2 * (ix + (iy - 1) * L1_) - 2 for ix in range(1, L1_ + 1) for iy in range(1, L2_ + 1)}
    out = []
    for sgn in (1.0, -1.0):                     # charge, then spin
        dens = nup + sgn * ndn                   # (Sa, Sb, site)
        stag = {c: dens[..., a] - dens[..., a + 1] for c, a in cells.items()}
        s0 = s1 = 0.0
        for (ix, iy), d1 in stag.items():
            for rx in range(1, L1_ + 1):
                for ry in range(1, L2_ + 1):
                    c2 = ((ix + rx - 1) % L1_ + 1, (iy + ry - 1) % L2_ + 1)
                    v = np.vdot(L1, d1 * stag[c2] * R1) / norm
                    s0 += v
                    s1 += np.cos(2 * np.pi / L1_ * rx + 2 * np.pi / L2_ * ry) * v
        out += [float(np.real(s0)) / Ns ** 2, float(np.real(s1)) / Ns ** 2]
    return out[0], out[1], out[2], out[3]


def tu_staggered_structure_factors(model):
    """Exact staggered charge and spin structure factors at (pi, pi) of the
    t-U sweep's measurement on a bipartite (square) lattice, the columns
    kdq_set_measure_full adds there: sum_ij e_i e_j <rho_i rho_j> / Ns^2 with
    e the two-colouring of the lattice, rho = n_up + n_dn (charge) or
    n_up - n_dn (spin), n_up = n_a, n_dn = 1 - n_b as in
    ``tu_structure_factors``.  Returns (charge, spin)."""
    import dqmc_oracle as O
    Ns = model.Ns
    if Ns > 12:
        raise ValueError(f"Fock-space sum needs Ns <= 12, got {Ns}")
    eps = O.staggered_signs(model.K).astype(np.float64)
    basis = _basis(Ns, Ns // 2)
    occ = _occupations(basis, Ns)
    m = occ[:, None, :] - occ[None, :, :]
    γ, η = np.asarray(model.γ), np.asarray(model.η)

    def V(l):
        f = {d: np.sum(γ * np.exp(1j * model.α[l - 1] * η * d)) for d in (-1, 0, 1)}
        return np.prod(np.select([m == -1, m == 0, m == 1], [f[-1], f[0], f[1]]), axis=2)

    R, L, _ = tu_states(model, V)
    Ha, Hb = gamma_op(model.HalfeK, basis), gamma_op(model.HalfeK.conj(), basis)
    Hia, Hib = gamma_op(model.HalfeKinv, basis), gamma_op(model.HalfeKinv.conj(), basis)
    R1 = Ha @ R @ Hb.T
    L1 = Hia.conj().T @ L @ Hib.conj()
    norm = np.vdot(L1, R1)
    nup = occ[:, None, :]
    ndn = 1.0 - occ[None, :, :]
    out = []
    for sgn in (1.0, -1.0):
        D = np.sum((nup + sgn * ndn) * eps, axis=2)     # sum_i e_i rho_i, (Sa, Sb)
        out.append(float(np.real(np.vdot(L1, D * D * R1) / norm)) / Ns ** 2)
    return out[0], out[1]
