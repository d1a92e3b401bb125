"""Host-side model construction: lattice, kinetic exponentials, trial state."""
import numpy as np
import pytest

import cases
from kapdqmc_gb300 import area_index, nnidx_F, nnK_Matrix, tUV_Hubbard_Para, xy_i
from kapdqmc_gb300.model import _nodes


def torus_adjacency(L):
    A = np.zeros((L * L, L * L))
    for x in range(L):
        for y in range(L):
            i = x + L * y
            for dx, dy in ((1, 0), (0, 1)):
                j = (x + dx) % L + L * ((y + dy) % L)
                A[i, j] = A[j, i] = 1
    return A


@pytest.mark.parametrize("L", [4, 8, 12])
def test_square45_is_the_LxL_torus(L):
    K = nnK_Matrix("SQUARE45", [L // 2, L])
    assert K.shape == (L * L, L * L)
    np.testing.assert_allclose(np.linalg.eigvalsh(K), np.linalg.eigvalsh(torus_adjacency(L)), atol=1e-10)


@pytest.mark.parametrize("L", [3, 6, 9])
def test_honeycomb_spectrum(L):
    K = nnK_Matrix("HoneyComb120", [L, L])
    k = 2 * np.pi * np.arange(L) / L
    e = []
    for k1 in k:
        for k2 in k:
            f = abs(1 + np.exp(1j * k1) + np.exp(1j * k2))
            e += [f, -f]
    np.testing.assert_allclose(np.linalg.eigvalsh(K), np.sort(e), atol=1e-10)


def test_bond_directions_are_perfect_matchings():
    for lat, site in (("HoneyComb120", [3, 3]), ("HoneyComb60", [3, 3]), ("SQUARE45", [2, 4])):
        nn = nnidx_F(lat, site)
        Ns = 2 * np.prod(site)
        for j in range(nn.shape[1]):
            ends = np.sort(nn[:, j, :].ravel())
            np.testing.assert_array_equal(ends, np.arange(1, Ns + 1))


def test_flux_hermitian_and_pi_flux_spectrum():
    K = nnK_Matrix("SQUARE90", [4, 4], flux=np.pi)
    assert np.linalg.norm(K - K.conj().T) < 1e-12


def test_kinetic_exponentials():
    m = cases.tu_square()
    np.testing.assert_allclose(m.eK @ m.eKinv, np.eye(m.Ns), atol=1e-12)
    np.testing.assert_allclose(m.HalfeK @ m.HalfeK, m.eK, atol=1e-12)


def test_trial_state_orthonormal():
    for m in (cases.tu_square(), cases.tu_honeycomb()):
        np.testing.assert_allclose(m.Pt.conj().T @ m.Pt, np.eye(m.ns), atol=1e-12)


def test_nodes_symmetric_and_ragged():
    np.testing.assert_array_equal(_nodes(100, 10), np.arange(0, 101, 10))
    assert _nodes(8, 3).tolist() == [0, 1, 4, 7, 8]
    assert _nodes(20, 8).tolist() == [0, 2, 10, 18, 20]


def test_nt_formulas():
    assert cases.c1().Nt == 100 and cases.c2().Nt == 400 and cases.c3().Nt == 320
    assert cases.c4().Nt == 200 and cases.c5().Nt == 200


def test_tuv_strict_stability_assert():
    with pytest.raises(AssertionError):
        tUV_Hubbard_Para(Ht=1.0, Hu=4.0, Hv=0.5, Lattice="SQUARE45", site=[4, 8], Δt=0.1, Θ=10.0,
                         BatchSize=10, Initial="H0")
    m = cases.c4()
    assert m.a == pytest.approx(1.0) and m.z == 4


def test_area_index_square45_left_half():
    # region A of the 8x8 torus: 32 sites
    idx = area_index("SQUARE45", [4, 8], ((1, 1), (4, 8)))
    assert len(idx) == 32 and len(set(idx)) == 32


def test_xy_i_range_check():
    with pytest.raises(ValueError):
        xy_i([3, 3], 4, 1)
