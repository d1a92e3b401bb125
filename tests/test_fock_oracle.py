"""The Fock-space machinery of oracle/fock_oracle.py on its own: the image of
a one-particle matrix is a representation, Slater overlaps are determinants,
and the hopping operators obey the fermionic algebra."""
import numpy as np

import fock_oracle as F


def test_gamma_is_a_representation_and_slater_overlaps_are_determinants():
    rng = np.random.default_rng(0)
    Ns, n = 6, 3
    basis = F._basis(Ns, n)
    A = rng.normal(size=(Ns, Ns)) + 1j * rng.normal(size=(Ns, Ns))
    B = rng.normal(size=(Ns, Ns))
    np.testing.assert_allclose(F.gamma_op(A @ B, basis), F.gamma_op(A, basis) @ F.gamma_op(B, basis),
                               rtol=1e-10, atol=1e-10)
    P = rng.normal(size=(Ns, n)) + 1j * rng.normal(size=(Ns, n))
    Q = rng.normal(size=(Ns, n))
    lhs = np.vdot(F.slater(P, basis), F.gamma_op(A, basis) @ F.slater(Q, basis))
    assert abs(lhs - np.linalg.det(P.conj().T @ A @ Q)) < 1e-9 * abs(lhs)


def test_hopping_operators_give_the_one_body_density_matrix():
    # for a Slater state, <c_i^dagger c_j> = (P (P^H P)^-1 P^H)_ji
    rng = np.random.default_rng(1)
    Ns, n = 6, 3
    basis = F._basis(Ns, n)
    P = rng.normal(size=(Ns, n))
    psi = F.slater(P, basis)
    rho = P @ np.linalg.inv(P.T @ P) @ P.T
    for i in range(Ns):
        for j in range(Ns):
            v = psi @ (F.hop_op(i, j, basis) @ psi) / (psi @ psi)
            assert abs(v - rho[j, i]) < 1e-10, (i, j)


def test_anticommutation_of_hops():
    # [c_i^dagger c_j, c_k^dagger c_l] = delta_jk c_i^dagger c_l - delta_il c_k^dagger c_j
    Ns, n = 5, 2
    basis = F._basis(Ns, n)
    E = {(i, j): F.hop_op(i, j, basis) for i in range(Ns) for j in range(Ns)}
    for (i, j, k, l) in [(0, 1, 1, 2), (2, 3, 0, 2), (1, 4, 4, 1), (3, 0, 0, 3)]:
        lhs = E[i, j] @ E[k, l] - E[k, l] @ E[i, j]
        rhs = (j == k) * E[i, l] - (i == l) * E[k, j]
        np.testing.assert_allclose(lhs, rhs, atol=1e-12)
