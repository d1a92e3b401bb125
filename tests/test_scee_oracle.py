"""The coupled SCEE sweep's CPU restatement (oracle/scee_oracle.py) against
brute-force Green's functions: after updates and node crossings in both
directions, each replica's G(tau,tau), G(tau0,tau0), G(tau,tau0) and
G(tau0,tau) equal those computed directly from its fields, and the
incrementally updated Grover inverse and determinant equal fresh ones."""
import numpy as np
import pytest

import cases
import dqmc_oracle as O
import philox
import scee_oracle as S
from kapdqmc_gb300 import Initial_s, area_index


def regions(m):
    L = m.site[1]
    A = area_index(m.Lattice, m.site, ([1, 1], [L // 3, L]))
    B = area_index(m.Lattice, m.site, ([1, 1], [L // 3, 2 * L // 3]))
    return A, B


def brute(sc, r, tau):
    m, s = sc.m, sc.s[r]
    sw = O._TUSweep(m, s, O.Tape([], []), False)

    def prod(t2, t1):
        M = np.eye(m.Ns, dtype=complex)
        for lt in range(t1 + 1, t2 + 1):
            M = sw.B_left(lt, M)
        return M

    t0 = sc.nodes[sc.Θ - 1]
    Gt, G0 = O.G_tau(m, s, tau), O.G_tau(m, s, t0)
    I = np.eye(m.Ns)
    if tau <= t0:
        return Gt, G0, -(I - Gt) @ np.linalg.inv(prod(t0, tau)), prod(t0, tau) @ Gt
    return Gt, G0, prod(tau, t0) @ G0, -(I - G0) @ np.linalg.inv(prod(tau, t0))


def check(sc, tau, tol=1e-9):
    for r in range(2):
        for got, ref in zip((sc.Gt[r], sc.G0[r], sc.Gt0[r], sc.G0t[r]), brute(sc, r, tau)):
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < tol
    for reg, det, inv in ((sc.A, sc.detA, sc.invA), (sc.B, sc.detB, sc.invB)):
        d, i = sc.grover(reg)
        assert abs(det - d) < 1e-9 * d
        assert np.linalg.norm(inv - i) < 1e-9 * np.linalg.norm(i)


@pytest.mark.parametrize("make", [cases.tu_honeycomb, cases.tu_quench])
def test_scee_state_matches_brute_force(make):
    m = make()
    A, B = regions(m)
    n = S.proposals_per_sweep(m)
    k, u = philox.tape(9, 0, 0, n)
    sc = S.SCEE(m, Initial_s(m, 1), Initial_s(m, 2), A, B, 0.5, 2, O.Tape(k, u)).init()
    check(sc, 0)
    half = m.Nt // 2
    for lt in range(1, half + 3):
        sc.forward_slice(lt)
        if lt in (2, half - 1, half + 2):
            check(sc, lt)
    for lt in range(half + 3, m.Nt + 1):
        sc.forward_slice(lt)
    for lt in range(m.Nt, 1, -1):
        sc.backward_slice(lt)
        if lt - 1 in (m.Nt - 1, half + 1, 3):
            check(sc, lt - 1)
    assert 0 < sum(sc.accepts) < len(sc.accepts)


def test_ratio_is_the_reweighted_weight_change():
    # the acceptance ratio of a replica-1 proposal equals the change of
    # W(s1) W(s2) |det g_A|^(2 lam) |det g_B|^(2 (1 - lam)) computed from scratch
    m = cases.tu_honeycomb()
    A, B = regions(m)
    lam = 0.3
    s1, s2 = Initial_s(m, 3), Initial_s(m, 4)
    sc = S.SCEE(m, s1, s2, A, B, lam, 1, O.Tape([1], [float("inf")])).init()   # u = inf: rejected, ratio only
    from kapdqmc_gb300.sweep import log_weight

    def total(ss):
        t = 0.0
        for s in ss:
            t += log_weight(m, s, O.log_det(m, s)[0])
        G0s = [O.G_tau(m, s, sc.nodes[sc.Θ - 1]) for s in ss]
        for reg, w in ((sc.A, lam), (sc.B, 1 - lam)):
            a, b = G0s[0][np.ix_(reg, reg)], G0s[1][np.ix_(reg, reg)]
            g = 2 * a @ b - a - b + np.eye(len(reg))
            t += 2 * w * np.log(abs(np.linalg.det(g)))
        return t

    lt, i = 1, 4
    for r in range(2):
        sc.wrap(r, lt, True)
    sold = int(sc.s[0][i, lt - 1])
    sx = O._sx(sold, 1)
    # ratio as the sweep computes it
    Δ = np.exp(1j * m.α[lt - 1] * (m.η[sx - 1] - m.η[sold - 1])) - 1
    pc = 1 + Δ * (1 - sc.Gt[0][i, i])
    rr = Δ / pc
    p = abs(pc) ** 2 * m.γ[sx - 1] / m.γ[sold - 1]
    for reg, inv, w in ((sc.A, sc.invA, lam), (sc.B, sc.invB, 1 - lam)):
        X = 2 * sc.G0[1][np.ix_(reg, reg)] - np.eye(len(reg))
        a = sc.G0t[0][reg, i] * rr
        b = (sc.Gt0[0][i, reg] @ X) @ inv
        p *= abs(1 + b @ a) ** (2 * w)
    s1n = sc.s[0].copy()
    s1n[i, lt - 1] = sx
    dw = total([s1n, sc.s[1]]) - total([sc.s[0], sc.s[1]])
    assert abs(dw - np.log(p)) < 1e-8, (dw, np.log(p))


def test_dop_state_and_ratio():
    # the disorder-operator sweep: state against brute force after updates and
    # node crossings, the incremental X inverses against fresh ones, and the
    # ratio against the reweighted weight change
    m = cases.tu_honeycomb()
    A, B = regions(m)
    alpha, lam = 0.7, 0.4
    n = 2 * m.Ns * m.Nt
    k, u = philox.tape(4, 0, 0, n)
    sc = S.DOP(m, Initial_s(m, 5), alpha, A, B, lam, 2, O.Tape(k, u)).init()
    half = m.Nt // 2
    for lt in range(1, half + 3):
        sc.forward_slice(lt)
    for r_check in (0,):
        for got, ref in zip((sc.Gt[0], sc.G0[0], sc.Gt0[0], sc.G0t[0]), brute(sc, 0, half + 2)):
            assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-9
    for reg, det, inv in ((sc.A, sc.detA, sc.invA), (sc.B, sc.detB, sc.invB)):
        d, i = sc.xmat(reg)
        assert abs(det - d) < 1e-9 * d
        assert np.linalg.norm(inv - i) < 1e-9 * np.linalg.norm(i)
    assert 0 < sum(sc.accepts) < len(sc.accepts)

    from kapdqmc_gb300.sweep import log_weight
    sc2 = S.DOP(m, Initial_s(m, 6), alpha, A, B, lam, 1, O.Tape([1], [float("inf")])).init()

    def total(s):
        t = log_weight(m, s, O.log_det(m, s)[0])
        G0 = O.G_tau(m, s, sc2.nodes[sc2.Θ - 1])
        e = np.exp(1j * alpha)
        for reg, w in ((sc2.A, lam), (sc2.B, 1 - lam)):
            X = (1 - e) * G0[np.ix_(reg, reg)] + e * np.eye(len(reg))
            t += 2 * w * np.log(abs(np.linalg.det(X)))
        return t

    lt, i = 1, 3
    sc2.wrap(0, lt, True)
    sold = int(sc2.s[0][i, lt - 1])
    sx = O._sx(sold, 1)
    Δ = np.exp(1j * m.α[lt - 1] * (m.η[sx - 1] - m.η[sold - 1])) - 1
    pc = 1 + Δ * (1 - sc2.Gt[0][i, i])
    rr = Δ / pc
    p = abs(pc) ** 2 * m.γ[sx - 1] / m.γ[sold - 1]
    e = np.exp(1j * alpha)
    for reg, inv, w in ((sc2.A, sc2.invA, lam), (sc2.B, sc2.invB, 1 - lam)):
        a = (1 - e) * (sc2.G0t[0][reg, i] * rr)
        b = sc2.Gt0[0][i, reg] @ inv
        p *= abs(1 + b @ a) ** (2 * w)
    s1 = sc2.s[0].copy()
    s1[i, lt - 1] = sx
    assert abs((total(s1) - total(sc2.s[0])) - np.log(p)) < 1e-8


def brute_tv(sc, r, tau):
    m, s = sc.m, sc.s[r]
    sw = O._TVSweep(m, s, O.Tape([], []), False)

    def prod(t2, t1):
        M = np.eye(m.Ns)
        for lt in range(t1 + 1, t2 + 1):
            M = sw.B_left(lt, M)
        return M

    t0 = sc.nodes[sc.Θ - 1]
    Gt, G0 = O.G_tau(m, s, tau), O.G_tau(m, s, t0)
    I = np.eye(m.Ns)
    if tau <= t0:
        return Gt, G0, -(I - Gt) @ np.linalg.inv(prod(t0, tau)), prod(t0, tau) @ Gt
    return Gt, G0, prod(tau, t0) @ G0, -(I - G0) @ np.linalg.inv(prod(tau, t0))


def test_scee_tv_state_and_ratio():
    m = cases.tv_honeycomb()
    A, B = regions(m)
    n = S.proposals_per_sweep_tv(m)
    k, u = philox.tape(9, 0, 0, n)
    sc = S.SCEE_TV(m, Initial_s(m, 1), Initial_s(m, 2), A, B, 0.5, 2, O.Tape(k, u)).init()
    half = m.Nt // 2
    for lt in range(1, m.Nt + 1):
        sc.forward_slice(lt)
        if lt in (3, half + 2):
            for r in range(2):
                for got, ref in zip((sc.Gt[r], sc.G0[r], sc.Gt0[r], sc.G0t[r]), brute_tv(sc, r, lt)):
                    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) < 1e-8
            for reg, det, inv in ((sc.A, sc.detA, sc.invA), (sc.B, sc.detB, sc.invB)):
                d, i = sc.grover(reg)
                assert abs(det - d) < 1e-8 * abs(d)
                assert np.linalg.norm(inv - i) < 1e-8 * np.linalg.norm(i)
    assert 0 < sum(sc.accepts) < len(sc.accepts)
    # ratio of a replica-1 proposal against the reweighted weight change
    lam = 0.3
    sc2 = S.SCEE_TV(m, Initial_s(m, 3), Initial_s(m, 4), A, B, lam, 1, O.Tape([1], [float("inf")])).init()
    from kapdqmc_gb300.sweep import log_weight

    def total(ss):
        t = sum(log_weight(m, s, O.log_det(m, s)[0]) for s in ss)
        G0s = [O.G_tau(m, s, sc2.nodes[sc2.Θ - 1]) for s in ss]
        for reg, w in ((sc2.A, lam), (sc2.B, 1 - lam)):
            a, b = G0s[0][np.ix_(reg, reg)], G0s[1][np.ix_(reg, reg)]
            t += w * np.log(abs(np.linalg.det(2 * a @ b - a - b + np.eye(len(reg)))))
        return t

    lt, j, i = 1, m.z - 1, 2
    for r in range(2):
        sc2.wrapK(r, True)
        sc2.wrapV(r, lt, j, True)
    sc2.propose_bond(0, lt, j, i)      # u = inf: rejected, the ratio is kept
    p = sc2.last_p
    s1 = sc2.s[0].copy()
    sold = int(s1[i, j, lt - 1])
    s1[i, j, lt - 1] = O._sx(sold, 1)
    dw = total([s1, sc2.s[1]]) - total(sc2.s)
    assert p > 0 and abs(dw - np.log(p)) < 1e-8, (dw, np.log(p))


@pytest.mark.parametrize("U", [4.0, -4.0])
def test_scee_tuv_state_matches_brute_force(U):
    m = cases.tuv_honeycomb(U=U)
    A, B = regions(m)
    n = 4 * m.Ns * m.z * m.Nt
    k, u = philox.tape(9, 0, 0, n)
    sc = S.SCEE_TUV(m, Initial_s(m, 1), Initial_s(m, 2), A, B, 0.5, 2, O.Tape(k, u)).init()
    for lt in range(1, m.Nt + 1):
        sc.forward_slice(lt)
    for lt in range(m.Nt, 7, -1):
        sc.backward_slice(lt)
    for r in range(2):
        s, sw = sc.s[r], O._TUVSweep(m, sc.s[r], O.Tape([], []), False)
        t0, tau = sc.nodes[sc.Θ - 1], 7
        Gt, G0 = O.G_tau(m, s, tau), O.G_tau(m, s, t0)
        M = np.eye(m.Ns, dtype=sc.I.dtype)
        for lt in range(tau + 1, t0 + 1):
            M = sw.B_left(lt, M)
        ref = (Gt, G0, -(np.eye(m.Ns) - Gt) @ np.linalg.inv(M), M @ Gt)
        for got, want in zip((sc.Gt[r], sc.G0[r], sc.Gt0[r], sc.G0t[r]), ref):
            assert np.linalg.norm(got - want) / np.linalg.norm(want) < 1e-9
    d, i = sc.grover(sc.A)
    assert abs(sc.detA - d) < 1e-9 * d
    assert 0 < sum(sc.accepts) < len(sc.accepts)
