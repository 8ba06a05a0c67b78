"""The 1D fast-diagonalization tables of the implicit solver's preconditioner
(advection_solver_implicit.cc:1020-1062), computed by the library's own
complex QR eigensolver, against numpy."""
import ctypes

import numpy as np
import pytest


def lib_tables(adv_lib, degree, alpha, sign_index):
    from advection_miniapp_gb300 import _lib
    n = degree + 1
    lam = np.zeros(2 * n)
    V = np.zeros(2 * n * n)
    VW = np.zeros(2 * n * n)
    A1 = np.zeros(n * n)
    res = ctypes.c_double()
    P = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    rc = _lib.load().adv_fdm_tables(degree, alpha, sign_index, P(lam), P(V), P(VW), P(A1), ctypes.byref(res))
    assert rc == 0
    c = lambda a: a[0::2] + 1j * a[1::2]
    return c(lam), c(V).reshape(n, n), c(VW).reshape(n, n), A1.reshape(n, n), res.value


def reference_1d(oracle_mod, degree, alpha, s):
    """W^{-1} A1 in the Lagrange basis on the Gauss points, from the oracle's points."""
    t = oracle_mod.tables(degree)
    gp, gw, n = t["gp"], t["gw"], degree + 1

    def lag(i, x):
        return np.prod([(x - gp[j]) / (gp[i] - gp[j]) for j in range(n) if j != i])

    def dlag(i, x):
        return sum(np.prod([(x - gp[j]) / (gp[i] - gp[j]) for j in range(n) if j not in (i, m)]) / (gp[i] - gp[m])
                   for m in range(n) if m != i)

    A = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            A[i, j] = (-dlag(i, gp[j]) * gw[j] - lag(i, 0.0) * lag(j, 0.0) * 0.5 * (1 - alpha * s)
                       + lag(i, 1.0) * lag(j, 1.0) * 0.5 * (1 + alpha * s)) / gw[i]
    return A, gw


@pytest.mark.parametrize("degree", range(1, 7))
@pytest.mark.parametrize("alpha", [1.0, 0.5])
@pytest.mark.parametrize("sign_index", [0, 1])
def test_fdm_tables_against_numpy(adv_lib, oracle_mod, degree, alpha, sign_index):
    lam, V, VW, A1, res = lib_tables(adv_lib, degree, alpha, sign_index)
    A, gw = reference_1d(oracle_mod, degree, alpha, 1.0 if sign_index == 0 else -1.0)
    np.testing.assert_allclose(A1, A, atol=1e-11 * np.abs(A).max())
    ref = np.linalg.eigvals(A)
    # same eigenvalues as numpy (as multisets)
    for l in lam:
        assert np.min(np.abs(ref - l)) <= 1e-9 * np.abs(ref).max()
    assert res < 1e-9
    # V Lambda V^{-1} = W^{-1} A1 and (V^{-1} W^{-1}) W = V^{-1}
    Vinv = VW @ np.diag(gw)
    np.testing.assert_allclose(V @ np.diag(lam) @ Vinv, A, atol=1e-9 * np.abs(A).max())
