"""Pins of the oracle's implicit-solver pieces (advection_solver_implicit.cc):
the mass matrix, vmult = c M - L, and the cellwise fast-diagonalization
preconditioner, which on an affine mesh with constant velocity must invert the
cell-local block of vmult exactly (the cell operator is then separable)."""
import numpy as np
import pytest

from test_fdm_tables import reference_1d


def numpy_fdm_tables(oracle_mod, degree, alpha):
    lams, Vs, VWs = [], [], []
    for s in (1.0, -1.0):
        A, gw = reference_1d(oracle_mod, degree, alpha, s)
        lam, V = np.linalg.eig(A)
        lams.append(lam)
        Vs.append(V)
        VWs.append(np.linalg.inv(V) @ np.diag(1.0 / gw))
    return np.array(lams), np.array(Vs), np.array(VWs)


def test_mass_matches_dense(oracle_mod):
    o = oracle_mod.Oracle(degree=3, n_cells=(2, 3, 2), mesh_type=1, deformation=0.07)
    u = np.random.default_rng(0).standard_normal(o.n_dofs)
    m = o.apply_mass(u)
    np.testing.assert_allclose(o.inverse_mass_dense(m), u, atol=1e-12)
    np.testing.assert_allclose(o.vmult(u, 3.0, 0.1), 3.0 * m - o.apply_unscaled(u, 0.1), atol=1e-13)


@pytest.mark.parametrize("degree,velocity", [(2, (1.0, 0.15, -0.05)), (4, (-0.3, 0.7, 0.4)), (3, (0.5, -1.0, 0.2))])
def test_fdm_inverts_the_cell_block_on_affine_meshes(oracle_mod, degree, velocity):
    o = oracle_mod.Oracle(degree=degree, n_cells=(3, 3, 3), velocity=velocity)
    n3 = (degree + 1) ** 3
    cm = 7.0
    tables = numpy_fdm_tables(oracle_mod, degree, 1.0)
    cell = 13  # an interior cell
    rng = np.random.default_rng(1)
    for _ in range(3):
        x = np.zeros(o.n_dofs)
        x[cell * n3:(cell + 1) * n3] = rng.standard_normal(n3)
        y = o.vmult(x, cm)
        r = np.zeros(o.n_dofs)
        r[cell * n3:(cell + 1) * n3] = y[cell * n3:(cell + 1) * n3]  # the cell-local block of vmult
        z = o.fdm_apply(tables, r, cm)
        np.testing.assert_allclose(z[cell * n3:(cell + 1) * n3], x[cell * n3:(cell + 1) * n3],
                                   atol=1e-11 * np.abs(x).max())
