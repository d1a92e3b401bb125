"""The coupled SCEE sweep in CUDA (through the C ABI) against the oracle's
restatement of ctrl_SCEEicr: identical accept sequences and fields for both
replicas of every pair, the per-sweep estimator rows and all four Green's
functions of each replica at the end."""
import numpy as np
import pytest

import cases
import dqmc_oracle as O
import philox
import scee_oracle as S
from kapdqmc_gb300 import Initial_s, area_index
from kapdqmc_gb300.sweep import Sweeper, ctrl_SCDOPicr, ctrl_SCEEicr

pytestmark = pytest.mark.gpu


def regions(m):
    L = m.site[1]
    return (area_index(m.Lattice, m.site, ([1, 1], [L // 3, L])),
            area_index(m.Lattice, m.site, ([1, 1], [L // 3, 2 * L // 3])))


def _tape(seed, pair, sweeps, n_rep):
    ks, us = [], []
    for w in range(sweeps):
        k0, u0 = philox.tape(seed, 2 * pair, w, n_rep)
        k1, u1 = philox.tape(seed, 2 * pair + 1, w, n_rep)
        ks.append(np.stack([k0, k1], axis=1).ravel())
        us.append(np.stack([u0, u1], axis=1).ravel())
    return O.Tape(np.concatenate(ks), np.concatenate(us))


@pytest.mark.parametrize("make,lam,nlam", [(cases.tu_honeycomb, 0.5, 2), (cases.tu_quench, 0.25, 3),
                                           (lambda: cases.tu_square(flux=np.pi), 1.0, 1)])
def test_scee_matches_oracle(make, lam, nlam):
    m = make()
    A, B = regions(m) if "HoneyComb" in m.Lattice else ([1, 2, 3, 4, 5, 6], [1, 2, 3])
    npairs, sweeps, seed = 2, 2, 31
    fields = np.stack([Initial_s(m, 70 + c) for c in range(2 * npairs)])
    n_rep = 2 * m.Ns * m.Nt
    with Sweeper(m, 2 * npairs) as sw:
        sw.set_fields(fields)
        sw.set_rng(seed)
        sw.enable_accept_log(n_rep * sweeps)
        sw.scee_enable(A, B, lam, nlam)
        Orows = sw.scee_run(sweeps)
        s_gpu = sw.get_fields()
        acc = sw.accept_log()
        Gs = [[sw.scee_green(c, w) for w in range(4)] for c in range(2 * npairs)]
    for p in range(npairs):
        ref = S.SCEE(m, fields[2 * p], fields[2 * p + 1], A, B, lam, nlam, _tape(seed, p, sweeps, n_rep)).run(sweeps)
        ra = np.array(ref.accepts).reshape(-1, 2)
        for r in range(2):
            np.testing.assert_array_equal(acc[2 * p + r].astype(bool), ra[:, r], err_msg=f"pair {p} replica {r}")
            np.testing.assert_array_equal(s_gpu[2 * p + r], ref.s[r])
            for w, G in enumerate((ref.Gt[r], ref.G0[r], ref.Gt0[r], ref.G0t[r])):
                rel = np.linalg.norm(Gs[2 * p + r][w] - G) / np.linalg.norm(G)
                assert rel < 1e-9, (p, r, w, rel)
        assert Orows[p, 0] == lam
        np.testing.assert_allclose(Orows[p, 1:], ref.O, rtol=1e-8)


def test_ctrl_scee_reference_shaped_call(tmp_path):
    m = cases.tu_honeycomb()
    A, B = regions(m)
    ss = [Initial_s(m, 1), Initial_s(m, 2)]
    out, O_ = ctrl_SCEEicr(str(tmp_path), m, A, B, 2, 0.5, 2, ss, True, seed=5)
    assert out.shape == (2,) + tuple(m.field_shape)
    assert O_.shape == (1, 3) and O_[0, 0] == 0.5
    files = list(tmp_path.iterdir())
    assert len(files) == 1 and files[0].name.startswith("tUSCEEHC120_t1.0U4.0size[3, 3]")


@pytest.mark.parametrize("make,alpha", [(cases.tu_honeycomb, 0.7), (cases.tu_quench, 1.9)])
def test_dop_matches_oracle(make, alpha):
    m = make()
    A, B = regions(m)
    nch, sweeps, seed, lam = 3, 2, 13, 0.4
    fields = np.stack([Initial_s(m, 90 + c) for c in range(nch)])
    n_rep = 2 * m.Ns * m.Nt
    with Sweeper(m, nch) as sw:
        sw.set_fields(fields)
        sw.set_rng(seed)
        sw.enable_accept_log(n_rep * sweeps)
        sw.dop_enable(alpha, A, B, lam, 2)
        Orows = sw.dop_run(sweeps)
        s_gpu = sw.get_fields()
        acc = sw.accept_log()
        Gs = [[sw.scee_green(c, w) for w in range(4)] for c in range(nch)]
    for c in range(nch):
        ks, us = zip(*(philox.tape(seed, c, w, n_rep) for w in range(sweeps)))
        ref = S.DOP(m, fields[c], alpha, A, B, lam, 2, O.Tape(np.concatenate(ks), np.concatenate(us))).run(sweeps)
        np.testing.assert_array_equal(acc[c].astype(bool), np.array(ref.accepts))
        np.testing.assert_array_equal(s_gpu[c], ref.s[0])
        for w, G in enumerate((ref.Gt[0], ref.G0[0], ref.Gt0[0], ref.G0t[0])):
            assert np.linalg.norm(Gs[c][w] - G) / np.linalg.norm(G) < 1e-9
        np.testing.assert_allclose(Orows[c, 1:], ref.O, rtol=1e-8)
    out, O_ = ctrl_SCDOPicr("", m, alpha, A, B, 1, lam, 2, fields[0], True, seed=1)
    assert out.shape == tuple(m.field_shape) and O_.shape == (1, 2)


def _tape_tv(seed, pair, sweeps, m):
    """Interleave the two replicas' bond streams in the t-V sweep's order:
    per slice and direction, bond by bond, replica 1 then replica 2."""
    nb, z, Nt = m.Ns // 2, m.z, m.Nt
    n_rep = 2 * nb * z * Nt
    ks, us = [], []
    for w in range(sweeps):
        k0, u0 = philox.tape(seed, 2 * pair, w, n_rep)
        k1, u1 = philox.tape(seed, 2 * pair + 1, w, n_rep)
        ks.append(np.stack([k0, k1], axis=1).ravel())
        us.append(np.stack([u0, u1], axis=1).ravel())
    return O.Tape(np.concatenate(ks), np.concatenate(us))


@pytest.mark.parametrize("make", [cases.tv_honeycomb, cases.tv_honeycomb60])
def test_scee_tv_matches_oracle(make):
    m = make()
    A, B = regions(m)
    npairs, sweeps, seed, lam, nlam = 2, 2, 17, 0.5, 2
    fields = np.stack([Initial_s(m, 50 + c) for c in range(2 * npairs)])
    n_rep = 2 * (m.Ns // 2) * m.z * m.Nt
    with Sweeper(m, 2 * npairs) as sw:
        sw.set_fields(fields)
        sw.set_rng(seed)
        sw.enable_accept_log(n_rep * sweeps)
        sw.scee_enable(A, B, lam, nlam)
        Orows = sw.scee_run(sweeps)
        s_gpu = sw.get_fields()
        acc = sw.accept_log()
        Gs = [[sw.scee_green(c, w) for w in range(4)] for c in range(2 * npairs)]
    for p in range(npairs):
        ref = S.SCEE_TV(m, fields[2 * p], fields[2 * p + 1], A, B, lam, nlam, _tape_tv(seed, p, sweeps, m)).run(sweeps)
        ra = np.array(ref.accepts).reshape(-1, 2)
        for r in range(2):
            np.testing.assert_array_equal(acc[2 * p + r].astype(bool), ra[:, r], err_msg=f"pair {p} replica {r}")
            np.testing.assert_array_equal(s_gpu[2 * p + r], ref.s[r])
            for w, G in enumerate((ref.Gt[r], ref.G0[r], ref.Gt0[r], ref.G0t[r])):
                rel = np.linalg.norm(Gs[2 * p + r][w] - G) / np.linalg.norm(G)
                assert rel < 1e-8, (p, r, w, rel)
        np.testing.assert_allclose(Orows[p, 1:], ref.O, rtol=1e-8)


def _tape_tuv(seed, pair, sweeps, m):
    n_rep = 2 * m.Ns * m.z * m.Nt
    ks, us = [], []
    for w in range(sweeps):
        k0, u0 = philox.tape(seed, 2 * pair, w, n_rep)
        k1, u1 = philox.tape(seed, 2 * pair + 1, w, n_rep)
        ks.append(np.stack([k0, k1], axis=1).ravel())
        us.append(np.stack([u0, u1], axis=1).ravel())
    return O.Tape(np.concatenate(ks), np.concatenate(us))


@pytest.mark.parametrize("make", [cases.tuv_honeycomb, lambda: cases.tuv_honeycomb(U=-4.0), cases.tuv_square])
def test_scee_tuv_matches_oracle(make):
    m = make()
    A, B = regions(m) if "HoneyComb" in m.Lattice else ([1, 2, 3, 4, 5, 6], [1, 2, 3])
    npairs, sweeps, seed, lam, nlam = 2, 2, 23, 0.5, 2
    fields = np.stack([Initial_s(m, 30 + c) for c in range(2 * npairs)])
    n_rep = 2 * m.Ns * m.z * m.Nt
    with Sweeper(m, 2 * npairs) as sw:
        sw.set_fields(fields)
        sw.set_rng(seed)
        sw.enable_accept_log(n_rep * sweeps)
        sw.scee_enable(A, B, lam, nlam)
        Orows = sw.scee_run(sweeps)
        s_gpu = sw.get_fields()
        acc = sw.accept_log()
        Gs = [[sw.scee_green(c, w) for w in range(4)] for c in range(2 * npairs)]
    for p in range(npairs):
        ref = S.SCEE_TUV(m, fields[2 * p], fields[2 * p + 1], A, B, lam, nlam, _tape_tuv(seed, p, sweeps, m)).run(sweeps)
        ra = np.array(ref.accepts).reshape(-1, 2)
        for r in range(2):
            np.testing.assert_array_equal(acc[2 * p + r].astype(bool), ra[:, r], err_msg=f"pair {p} replica {r}")
            np.testing.assert_array_equal(s_gpu[2 * p + r], ref.s[r])
            for w, G in enumerate((ref.Gt[r], ref.G0[r], ref.Gt0[r], ref.G0t[r])):
                rel = np.linalg.norm(Gs[2 * p + r][w] - G) / np.linalg.norm(G)
                assert rel < 1e-9, (p, r, w, rel)
        np.testing.assert_allclose(Orows[p, 1:], ref.O, rtol=1e-8)
