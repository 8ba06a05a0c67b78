"""Implicit path on the GPU against the oracle: the operator M/dt + A
(vmult), the mass matrix, the block-Jacobi FDM preconditioner, FGMRES (its
residual re-checked by the oracle) and BDF2 steps with the preconditioner in
FP64 and FP32."""
import numpy as np
import pytest

from test_oracle_implicit import numpy_fdm_tables

pytestmark = pytest.mark.gpu

CASES = {
    "curved-k4": dict(degree=4, n_cells=(4, 3, 4), mesh_type=1, deformation=0.08),
    "affine-k3": dict(degree=3, n_cells=(3, 4, 3), velocity=(-0.3, 0.7, 0.4)),
    "affine-k2-dirichlet": dict(degree=2, n_cells=(3, 3, 3), periodic=0, boundary_value=0),
    "rotating-k3": dict(degree=3, n_cells=(3, 3, 3), periodic=0, velocity_type=1, velocity=(1.0, 1.0, 0.3),
                        velocity_period=0.5, initial_condition=1, ic_params=(0.3, 0.5, 0.5, 0.2), boundary_value=0),
}


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rel(a, b):
    a = a.cpu().numpy() if hasattr(a, "cpu") else a
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("case", sorted(CASES))
def test_vmult_and_mass(cuda, oracle_mod, adv_lib, case):
    torch = cuda
    o = oracle_mod.Oracle(**CASES[case])
    g = adv_lib.AdvectionOperation(**CASES[case])
    u = np.random.default_rng(3).standard_normal(o.n_dofs)
    d = g.initialize_dof_vector()
    g.apply_mass(dev(torch, u), d)
    assert rel(d, o.apply_mass(u)) <= 1e-13
    for cm, t in ((12.5, 0.0), (3.0, 0.4)):
        g.vmult(dev(torch, u), d, cm, t)
        assert rel(d, o.vmult(u, cm, t)) <= 1e-12


@pytest.mark.parametrize("case", ["curved-k4", "affine-k3", "rotating-k3"])
@pytest.mark.parametrize("precision", [0, 1])
def test_fdm_preconditioner(cuda, oracle_mod, adv_lib, case, precision):
    torch = cuda
    cfg = CASES[case]
    o = oracle_mod.Oracle(**cfg)
    g = adv_lib.AdvectionOperation(**cfg)
    s = adv_lib.ImplicitSolver(g, restart=4, precond_precision=precision)
    r = np.random.default_rng(4).standard_normal(o.n_dofs)
    ref = o.fdm_apply(numpy_fdm_tables(oracle_mod, cfg["degree"], 1.0), r, 9.0)
    d = g.initialize_dof_vector()
    s.precondition(dev(torch, r), d, 9.0, 0.0)
    # FP32: round-off amplified by the condition number of the complex
    # eigenvector matrices (about 1e4 at degree 4); FGMRES is flexible and
    # absorbs it (see the BDF2 test: FP32- and FP64-preconditioned solutions agree)
    assert rel(d, ref) <= (1e-10 if precision == 0 else 2e-3)


@pytest.mark.parametrize("precision", [0, 1])
def test_fgmres_residual_checked_by_oracle(cuda, oracle_mod, adv_lib, precision):
    torch = cuda
    cfg = CASES["curved-k4"]
    o = oracle_mod.Oracle(**cfg)
    g = adv_lib.AdvectionOperation(**cfg)
    s = adv_lib.ImplicitSolver(g, restart=10, precond_precision=precision)
    dt = 8 * o.time_step(1.0) * 0.5
    cm = 1.5 / dt
    b = o.apply_mass(np.random.default_rng(5).standard_normal(o.n_dofs))
    x = g.initialize_dof_vector()
    its, res = s.fgmres(cm, 0.0, dev(torch, b), x, rel_tol=1e-10, max_iterations=500)
    xs = x.cpu().numpy()
    true_res = np.linalg.norm(b - o.vmult(xs, cm)) / np.linalg.norm(b)
    assert res <= 1e-10 and true_res <= 2e-10, (its, res, true_res)
    assert its < 200


def test_bdf2_steps_and_preconditioner_precision(cuda, oracle_mod, adv_lib):
    """BDF2 at Courant 8 on a small curved mesh: every step solves its system
    (checked by the oracle), FP32 and FP64 preconditioners give the same
    solution to the solver tolerance."""
    torch = cuda
    cfg = dict(degree=4, n_cells=(6, 6, 6), mesh_type=1, deformation=0.08)
    o = oracle_mod.Oracle(**cfg)
    g = adv_lib.AdvectionOperation(**cfg)
    dt = g.time_step(8.0)
    finals, iters = {}, {}
    for precision in (0, 1):
        s = adv_lib.ImplicitSolver(g, restart=30, precond_precision=precision)
        u_nm1 = g.initialize_dof_vector()
        u_n = g.initialize_dof_vector()
        g.project_initial(u_n)
        u_new = g.initialize_dof_vector()
        its = []
        for step in range(6):
            its.append(s.bdf2_step((step + 1) * dt, dt, step == 0, u_n, u_nm1, u_new, rel_tol=1e-10))
            if step == 2:
                # the oracle re-checks this step's linear system
                un, unm1, unew = u_n.cpu().numpy(), u_nm1.cpu().numpy(), u_new.cpu().numpy()
                cm = 1.5 / dt
                b = o.apply_mass((2.0 * un - 0.5 * unm1) / dt)
                assert np.linalg.norm(b - o.vmult(unew, cm)) / np.linalg.norm(b) <= 2e-10
            u_nm1, u_n, u_new = u_n, u_new, u_nm1
        finals[precision] = u_n.cpu().numpy()
        iters[precision] = its
    assert rel(finals[1], finals[0]) <= 1e-8, iters


def run_bdf2(adv_lib, g, dt, steps):
    s = adv_lib.ImplicitSolver(g, restart=30, precond_precision=1)
    u_nm1, u_n, u_new = (g.initialize_dof_vector() for _ in range(3))
    g.project_initial(u_n)
    for step in range(steps):
        s.bdf2_step((step + 1) * dt, dt, step == 0, u_n, u_nm1, u_new, rel_tol=1e-11)
        u_nm1, u_n, u_new = u_n, u_new, u_nm1
    err, nrm = g.l2_error(u_n, steps * dt)
    return err / nrm


def test_bdf2_second_order_in_time(cuda, adv_lib):
    """Halving dt at fixed final time cuts the error by about 4 (spatial error
    well below the temporal one: 8^3 cells of degree 5)."""
    g = adv_lib.AdvectionOperation(degree=5, n_cells=(8, 8, 8), mesh_type=1, deformation=0.08)
    dt = g.time_step(2.0)
    e1 = run_bdf2(adv_lib, g, dt, 8)
    e2 = run_bdf2(adv_lib, g, dt / 2, 16)
    assert e1 / e2 > 3.2, (e1, e2)


@pytest.mark.parametrize("case", ["curved-k4", "rotating-k3", "affine-k2-dirichlet"])
def test_bdf2_step_equals_nodal_fgmres_solve(cuda, oracle_mod, adv_lib, case):
    """adv_bdf2_step solves on the Gauss-point basis (values at the Gauss
    points, residuals as dual coefficients there, the collocation-form
    operator and the FDM preconditioner without its basis transforms) and
    stops on the nodal residual.  Its implicit-Euler and BDF2 steps equal a
    nodal FGMRES solve (adv_fgmres) of the same systems, and the oracle
    confirms the nodal residuals."""
    cfg = CASES[case]
    o = oracle_mod.Oracle(**cfg)
    g = adv_lib.AdvectionOperation(**cfg)
    s = adv_lib.ImplicitSolver(g, restart=30, precond_precision=0)
    dt = g.time_step(4.0)
    u0 = g.initialize_dof_vector()
    g.project_initial(u0)
    u1, u2 = g.initialize_dof_vector(), g.initialize_dof_vector()
    s.bdf2_step(dt, dt, True, u0, None, u1, rel_tol=1e-12)
    s.bdf2_step(2 * dt, dt, False, u1, u0, u2, rel_tol=1e-12)
    # the same systems through the nodal solver
    m0, x1 = g.initialize_dof_vector(), u0.clone()
    g.apply_mass(u0 / dt, m0)
    s.fgmres(1.0 / dt, dt, m0, x1, rel_tol=1e-12, max_iterations=2000)
    assert rel(u1, x1.cpu().numpy()) <= 1e-9
    m1, x2 = g.initialize_dof_vector(), 2 * u1 - u0
    g.apply_mass((2.0 * u1 - 0.5 * u0) / dt, m1)
    s.fgmres(1.5 / dt, 2 * dt, m1, x2, rel_tol=1e-12, max_iterations=2000)
    assert rel(u2, x2.cpu().numpy()) <= 1e-9
    for unew, cm, rhs, t in ((u1, 1.0 / dt, u0.cpu().numpy() / dt, dt),
                             (u2, 1.5 / dt, (2.0 * u1.cpu().numpy() - 0.5 * u0.cpu().numpy()) / dt, 2 * dt)):
        b = o.apply_mass(rhs)
        assert np.linalg.norm(b - o.vmult(unew.cpu().numpy(), cm, t)) / np.linalg.norm(b) <= 2e-12
