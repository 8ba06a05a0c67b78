"""The oracle's 1D tables against numpy/scipy (Gauss, Gauss-Lobatto, Lagrange basis)."""
import numpy as np
import pytest
from numpy.polynomial import legendre as L


@pytest.mark.parametrize("degree", range(1, 7))
def test_gauss_points_and_weights(oracle_mod, degree):
    t = oracle_mod.tables(degree)
    x, w = L.leggauss(degree + 1)
    np.testing.assert_allclose(t["gp"], (x + 1) / 2, atol=1e-15, rtol=0)
    np.testing.assert_allclose(t["gw"], w / 2, atol=1e-15, rtol=0)


@pytest.mark.parametrize("degree", range(1, 7))
def test_gauss_lobatto_nodes(oracle_mod, degree):
    t = oracle_mod.tables(degree)
    # interior GL nodes: roots of P_k'
    interior = np.sort(L.legroots(L.legder([0] * degree + [1]))) if degree > 1 else np.array([])
    ref = np.concatenate([[0.0], (interior + 1) / 2, [1.0]])
    np.testing.assert_allclose(t["gl"], ref, atol=1e-14, rtol=0)


@pytest.mark.parametrize("degree", range(1, 7))
def test_lagrange_matrices(oracle_mod, degree):
    t = oracle_mod.tables(degree)
    n = degree + 1
    gl, gp = t["gl"], t["gp"]
    # S[q, i] = phi_i(g_q) for the Lagrange basis on the GL nodes
    V = np.vander(gl, n, increasing=True)
    coef = np.linalg.solve(V, np.eye(n))  # column i: monomial coefficients of phi_i
    S = np.vander(gp, n, increasing=True) @ coef
    dV = np.zeros((n, n))
    for p in range(1, n):
        dV[:, p] = p * gp ** (p - 1)
    D = dV @ coef
    np.testing.assert_allclose(t["S"], S, atol=1e-12)
    np.testing.assert_allclose(t["D"], D, atol=1e-10)
    np.testing.assert_allclose(t["Sinv"] @ t["S"], np.eye(n), atol=1e-12)
    # quadrature with n Gauss points integrates phi_i phi_j exactly
    M_exact = np.zeros((n, n))
    xq, wq = L.leggauss(n + 2)
    Sq = np.vander((xq + 1) / 2, n, increasing=True) @ coef
    M_exact = Sq.T @ np.diag(wq / 2) @ Sq
    np.testing.assert_allclose(t["S"].T @ np.diag(t["gw"]) @ t["S"], M_exact, atol=1e-14)


def test_lsrk_coefficients_consistency(oracle_mod):
    # the classical order conditions of the 2N-storage schemes: sum b = 1
    for scheme, order in [(0, 3), (1, 4), (2, 4), (3, 5)]:
        a, b = oracle_mod.lsrk_coefficients(scheme)
        assert len(a) == len(b) - 1
        assert abs(b.sum() - 1.0) < 1e-12
