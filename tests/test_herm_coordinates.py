"""The Hermitian-coordinate form of the k-pair contraction, checked in numpy on random operators.

The column-block kernels (csrc/dmd_pairs_cb.cuh) store Q1 = M^H P1 M and Q2 = M^T P2 conj(M), take
the real coordinates r, s of rt = conj(D) o rho and st = conj(D) o (1 - rho), and accumulate
X' = M^H X, Y' = M^H Y; the finish maps them back. These identities hold for any complex P and
any Hermitian rho; a non-Hermitian rho is split into H + i A and contracted twice.
"""
import numpy as np
import pytest


def m_matrix(nb):
    """v = M q: q[(i,i)] = v_ii; i < j: q[(i,j)] = Re v_ij, q[(j,i)] = Im v_ij."""
    n2 = nb * nb
    M = np.zeros((n2, n2), complex)
    for p1 in range(nb):
        for p2 in range(nb):
            j = p1 * nb + p2
            if p1 == p2:
                M[j, j] = 1
            elif p1 < p2:
                M[j, j] = 1
                M[p2 * nb + p1, j] = 1
            else:
                M[p2 * nb + p1, j] = 1j
                M[j, j] = -1j
    return M


def coords(v, nb):
    """real coordinates of a Hermitian matrix given as its (nb*nb) vector"""
    V = v.reshape(nb, nb)
    q = np.zeros((nb, nb))
    for i in range(nb):
        q[i, i] = V[i, i].real
        for j in range(i + 1, nb):
            q[i, j] = V[i, j].real
            q[j, i] = V[i, j].imag
    return q.reshape(-1)


def back(xp, nb):
    """X = (M^H)^-1 X' as the finish kernel forms it"""
    X = xp.reshape(nb, nb).copy()
    for i in range(nb):
        for j in range(i + 1, nb):
            u, l = xp[i * nb + j], xp[j * nb + i]
            X[i, j] = 0.5 * (u + 1j * l)
            X[j, i] = 0.5 * (u - 1j * l)
    return X.reshape(-1)


def rand_herm(rng, nb):
    A = rng.standard_normal((nb, nb)) + 1j * rng.standard_normal((nb, nb))
    return 0.5 * (A + A.conj().T)


@pytest.mark.parametrize("nb", [1, 2, 3, 4])
def test_transformed_contraction_equals_complex_form(nb):
    rng = np.random.default_rng(nb)
    n2 = nb * nb
    M = m_matrix(nb)
    P1 = rng.standard_normal((n2, n2)) + 1j * rng.standard_normal((n2, n2))
    P2 = rng.standard_normal((n2, n2)) + 1j * rng.standard_normal((n2, n2))
    Q1 = M.conj().T @ P1 @ M
    Q2 = M.T @ P2 @ M.conj()
    rt_c, st_c, rt_k, st_k = (rand_herm(rng, nb).reshape(-1) for _ in range(4))
    # complex form (kernel contract): forward row k from column c, reverse column c from row k
    X_k = P1 @ rt_c
    Y_k = P2.T @ st_c
    Y_c = P1.conj().T @ st_k
    X_c = P2.conj() @ rt_k
    r_c, s_c, r_k, s_k = coords(rt_c, nb), coords(st_c, nb), coords(rt_k, nb), coords(st_k, nb)
    np.testing.assert_allclose(M @ r_c, rt_c, atol=1e-14)
    np.testing.assert_allclose(back(Q1 @ r_c, nb), X_k, atol=1e-12)
    np.testing.assert_allclose(back(Q2.T @ s_c, nb), Y_k, atol=1e-12)
    np.testing.assert_allclose(back(Q1.conj().T @ s_k, nb), Y_c, atol=1e-12)
    np.testing.assert_allclose(back(Q2.conj() @ r_k, nb), X_c, atol=1e-12)


def test_non_hermitian_state_as_two_passes():
    nb = 2
    rng = np.random.default_rng(7)
    M = m_matrix(nb)
    P1 = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    Q1 = M.conj().T @ P1 @ M
    V = rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))
    H = 0.5 * (V + V.conj().T)
    A = (V - V.conj().T) / 2j
    np.testing.assert_allclose(H + 1j * A, V, atol=1e-15)
    xp = Q1 @ coords(H.reshape(-1), nb) + 1j * (Q1 @ coords(A.reshape(-1), nb))
    np.testing.assert_allclose(back(xp, nb), P1 @ V.reshape(-1), atol=1e-12)

