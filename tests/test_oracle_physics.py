"""Self-made pins of the CPU oracle (the reference ships no tests or golden data).

* every term of the sum-factorized operator against a dense-matrix
  implementation (basis evaluated at all 3D points, Cholesky mass solve);
* spatial convergence against the analytic solution, mass conservation,
  energy decay of the upwind flux, consistency of the spatial operator with
  -a . grad u (the ExactSolutionTimeDer idea, advection_solver.cc:187-225);
* the temporal order of the LSRK schemes and the reference's aliasing
  patterns of perform_stage (advection_solver.cc:917-936).
"""
import numpy as np
import pytest

CASES = {
    "affine-periodic-k3": dict(degree=3, n_cells=(3, 3, 3)),
    "affine-periodic-k1": dict(degree=1, n_cells=(3, 2, 4)),
    "affine-periodic-k6": dict(degree=6, n_cells=(2, 2, 2)),
    "curved-periodic-k4": dict(degree=4, n_cells=(3, 3, 3), mesh_type=1, deformation=0.08),
    "curved-dirichlet-k2": dict(degree=2, n_cells=(3, 2, 2), mesh_type=1, deformation=0.06, periodic=0,
                                initial_condition=2),
    "affine-dirichlet-k3-skew": dict(degree=3, n_cells=(2, 3, 2), periodic=0, factor_skew=0.5,
                                     initial_condition=2),
    "affine-central-k2": dict(degree=2, n_cells=(3, 3, 3), flux_alpha=0.0),
    "rotating-dirichlet-k3": dict(degree=3, n_cells=(3, 3, 2), periodic=0, velocity_type=1,
                                  velocity=(1.0, 1.0, 0.3), velocity_period=0.5, initial_condition=1,
                                  ic_params=(0.3, 0.5, 0.5, 0.1), boundary_value=0),
    "sipg-dirichlet-k3": dict(degree=3, n_cells=(3, 2, 2), periodic=0, velocity_type=1,
                              velocity=(1.0, 1.0, 0.3), velocity_period=0.5, diffusion=1e-2,
                              penalty_factor=1.0, initial_condition=1, ic_params=(0.3, 0.5, 0.5, 0.2),
                              boundary_value=0),
    "sipg-periodic-curved-k2": dict(degree=2, n_cells=(3, 3, 3), mesh_type=1, deformation=0.05,
                                    diffusion=3e-2),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_sum_factorization_matches_dense(oracle_mod, case):
    o = oracle_mod.Oracle(**CASES[case])
    rng = np.random.default_rng(1)
    u = rng.standard_normal(o.n_dofs)
    for t in (0.0, 0.37):
        a = o.apply_unscaled(u, t)
        b = o.apply_unscaled_dense(u, t)
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
    m1, m2 = o.inverse_mass(u), o.inverse_mass_dense(u)
    assert np.abs(m1 - m2).max() <= 1e-12 * np.abs(m2).max()


def run(o, steps, dt, scheme=1):
    u = o.project(0.0)
    r, k = o.zeros(), o.zeros()
    t = 0.0
    for _ in range(steps):
        o.lsrk_step(t, dt, u, r, k, scheme)
        t += dt
    return u, t


@pytest.mark.parametrize("mesh_type", [0, 1])
def test_spatial_convergence(oracle_mod, mesh_type):
    errs = []
    for n in (4, 8):
        o = oracle_mod.Oracle(degree=3, n_cells=(n, n, n), mesh_type=mesh_type, deformation=0.08)
        dt = o.time_step(0.5)
        steps = int(round(0.2 / dt))
        u, t = run(o, steps, 0.2 / steps)
        err, nrm = o.l2_error(u, t)
        errs.append(err / nrm)
    rate = np.log2(errs[0] / errs[1])
    assert rate > 3.5, (errs, rate)


def test_conservation_and_energy(oracle_mod):
    o = oracle_mod.Oracle(degree=3, n_cells=(4, 4, 4), mesh_type=1, deformation=0.08)
    dt = o.time_step(0.5)
    u = o.project(0.0)
    r, k = o.zeros(), o.zeros()
    m0 = o.mass_energy(u)
    e_prev = m0[1]
    for s in range(10):
        o.lsrk_step(s * dt, dt, u, r, k)
        me = o.mass_energy(u)
        assert abs(me[0] - m0[0]) < 1e-13
        assert me[1] <= e_prev * (1 + 1e-14)
        e_prev = me[1]


def test_operator_consistency_with_exact_derivative(oracle_mod):
    # M^{-1} L applied to the interpolated smooth wave approximates -a . grad u
    errs = []
    for n in (4, 8):
        o = oracle_mod.Oracle(degree=4, n_cells=(n, n, n), initial_condition=2)
        u = o.project(0.0)
        du = o.apply(u, 0.0)
        # exact time derivative at the support points by a centred difference in time of u(x - a t)
        eps = 1e-5
        ref = (o.interpolate(eps) - o.interpolate(-eps)) / (2 * eps)
        errs.append(np.sqrt(np.mean((du - ref) ** 2)) / np.sqrt(np.mean(ref ** 2)))
    assert np.log2(errs[0] / errs[1]) > 2.5, errs


@pytest.mark.parametrize("scheme,order", [(0, 3), (1, 4), (2, 4), (3, 5)])
def test_lsrk_temporal_order(oracle_mod, scheme, order):
    o = oracle_mod.Oracle(degree=2, n_cells=(2, 2, 2), initial_condition=2)
    T = 0.2

    def solve(steps, sch):
        u = o.project(0.0)
        r, k = o.zeros(), o.zeros()
        dt = T / steps
        for s in range(steps):
            o.lsrk_step(s * dt, dt, u, r, k, sch)
        return u

    ref = solve(400, 3)
    e1 = np.abs(solve(10, scheme) - ref).max()
    e2 = np.abs(solve(20, scheme) - ref).max()
    assert np.log2(e1 / e2) > order - 0.4, (e1, e2)


def test_perform_stage_aliasing_patterns(oracle_mod):
    o = oracle_mod.Oracle(degree=3, n_cells=(3, 3, 3), mesh_type=1, deformation=0.08)
    rng = np.random.default_rng(3)
    u0 = rng.standard_normal(o.n_dofs)
    r0 = rng.standard_normal(o.n_dofs)
    b, a, t = 0.013, 0.021, 0.3
    k_ref = o.apply(r0, t)
    # first-stage pattern: r_in == u, k == r_out
    u = u0.copy()
    r = o.zeros()
    o.perform_stage(t, b, a, u, r, u, r)
    k0 = o.apply(u0, t)
    np.testing.assert_allclose(u, u0 + b * k0, rtol=0, atol=1e-13)
    np.testing.assert_allclose(r, u0 + a * k0, rtol=0, atol=1e-13)
    # later-stage pattern: r_in == r_out, separate k
    u = u0.copy()
    r = r0.copy()
    k = o.zeros()
    o.perform_stage(t, b, a, r, k, u, r)
    np.testing.assert_allclose(u, u0 + b * k_ref, rtol=0, atol=1e-13)
    np.testing.assert_allclose(r, u0 + a * k_ref, rtol=0, atol=1e-13)
    # last stage: a == 0 updates only u; the inverse-mass cell_loop still
    # leaves k in next_ri (advection_solver.cc:722-740)
    u = u0.copy()
    r = r0.copy()
    o.perform_stage(t, b, 0.0, r, k, u, r)
    np.testing.assert_allclose(u, u0 + b * k_ref, rtol=0, atol=1e-13)
    np.testing.assert_allclose(r, k_ref, rtol=0, atol=1e-13)


def test_time_step_rule(oracle_mod):
    # advection_solver.cc:1163-1165 on the 8^3 affine workload: h = 1/8, |a| = sqrt(1.025), k = 3
    o = oracle_mod.Oracle(degree=3, n_cells=(8, 8, 8))
    expected = 0.5 * 0.125 / np.sqrt(1.0 + 0.15 ** 2 + 0.05 ** 2) / 3 ** 1.5
    assert abs(o.time_step(0.5) - expected) < 1e-15
    assert abs(expected - 0.0118805) < 1e-6


def test_time_step_with_diffusion_is_stable(oracle_mod):
    """The diffusive limit: 4^3 cells of degree 5 with nu = 8e-3 have the
    ratio of diffusive to advective stiffness (proportional to nu / h) of the
    32^3 advection-diffusion workload with nu = 1e-3; with the combined rule
    the energy decays over 60 steps (the advective rule alone reaches 1e29
    within 20 steps)."""
    cfg = dict(degree=5, n_cells=(4, 4, 4), periodic=0, velocity_type=1, velocity=(1.0, 1.0, 0.3),
               velocity_period=0.5, diffusion=8e-3, initial_condition=1, ic_params=(0.3, 0.5, 0.5, 0.2),
               boundary_value=0)
    o = oracle_mod.Oracle(**cfg)
    h, k1, nu = 0.25, 6.0, 8e-3
    dt_a = 0.5 * h / np.sqrt(2.09) / 5 ** 1.5
    dt_d = 0.3 * h * h / (nu * k1 ** 4)
    dt = o.time_step(0.5)
    assert abs(dt - 1.0 / (1.0 / dt_a + 1.0 / dt_d)) <= 1e-15 * dt
    u = o.project(0.0)
    r, k = o.zeros(), o.zeros()
    e0 = o.mass_energy(u)[1]
    for s in range(60):
        o.lsrk_step(s * dt, dt, u, r, k)
    assert np.isfinite(u).all() and o.mass_energy(u)[1] < e0
