"""Slab-partitioned operator on one GPU: the slabs of a partition, with their
ghost layers exchanged between stages, reproduce the whole-mesh operator bit
for bit (apply, LSRK stages, projection) and its diagnostics to round-off.
The slabs run one after another; no kernel waits on another."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    "curved-k4": dict(degree=4, n_cells=(3, 4, 5), mesh_type=1, deformation=0.08),
    "curved-k3-fp32": dict(degree=3, n_cells=(4, 3, 5), mesh_type=1, deformation=0.08, precision=1),
    "affine-k3-dirichlet-skew": dict(degree=3, n_cells=(3, 3, 4), periodic=0, velocity=(0.4, -0.3, 0.8),
                                     factor_skew=0.5),
    "sipg-k2-rotating": dict(degree=2, n_cells=(4, 4, 4), periodic=0, velocity_type=1, velocity=(1.0, 1.0, 0.3),
                             velocity_period=0.5, diffusion=2e-3, initial_condition=1,
                             ic_params=(0.3, 0.5, 0.5, 0.2), boundary_value=0),
    "affine-k5-uniform": dict(degree=5, n_cells=(2, 2, 3)),
}


class StageLoop:
    """Whole-mesh operator driven through the reference's stage loop."""

    def __init__(self, op):
        self.op = op

    def perform_stage(self, *a, **k):
        self.op.perform_stage(*a, **k)


@pytest.mark.parametrize("n_slabs", [2, 3])
@pytest.mark.parametrize("case", sorted(CASES))
def test_slabs_reproduce_whole_mesh(cuda, adv_lib, case, n_slabs):
    torch = cuda
    from advection_miniapp_gb300.distributed import SlabGroup
    cfg = adv_lib.make_config(**CASES[case])
    if cfg.n_cells[2] < n_slabs:
        pytest.skip("fewer layers than slabs")
    whole = adv_lib.AdvectionOperation(cfg)
    grp = SlabGroup(cfg, n_slabs)
    u = torch.from_numpy(np.random.default_rng(1).standard_normal(whole.n_dofs)).cuda()
    d = whole.initialize_dof_vector()
    whole.apply(u, d, 0.3)
    us = [lay.from_global(u) for lay in grp.layouts]
    for lay, v in zip(grp.layouts, us):  # stale ghosts: the exchange must overwrite them
        v[:lay.owned_begin] = 7.0
        v[lay.owned_begin + lay.owned_dofs:] = -7.0
    ds = grp.initialize_dof_vector()
    grp.apply(us, ds, 0.3)
    assert torch.equal(grp.to_global(ds), d)

    # projection, then LSRK(5,4) steps through the stage loop on both
    integ = adv_lib.LowStorageRungeKuttaIntegrator(adv_lib.LSRK_5_4)
    dt = whole.time_step(0.5)
    assert grp.time_step(0.5) == dt
    uw, rw, kw = (whole.initialize_dof_vector() for _ in range(3))
    whole.project_initial(uw)
    ug, rg, kg = grp.initialize_dof_vector(), grp.initialize_dof_vector(), grp.initialize_dof_vector()
    grp.project_initial(ug)
    assert torch.equal(grp.to_global(ug), uw)
    for step in range(3):
        integ.perform_time_step(StageLoop(whole), step * dt, dt, uw, rw, kw)
        integ.perform_time_step(grp, step * dt, dt, ug, rg, kg)
    assert torch.equal(grp.to_global(ug), uw)
    ew, nw = whole.l2_error(uw, 3 * dt)
    eg, ng = grp.l2_error(ug, 3 * dt)
    assert abs(eg - ew) <= 1e-13 * ew and abs(ng - nw) <= 1e-13 * nw
    mw, mg = whole.compute_mass_and_energy(uw), grp.compute_mass_and_energy(ug)
    assert np.allclose(mg, mw, rtol=1e-12, atol=1e-14 * np.abs(mw).max())
    grp.close()


def test_single_rank_distributed_operator(cuda, adv_lib):
    """One rank on a periodic mesh exchanges with itself (no process group)."""
    torch = cuda
    from advection_miniapp_gb300.distributed import DistributedAdvectionOperation
    cfg = adv_lib.make_config(**CASES["curved-k4"])
    whole = adv_lib.AdvectionOperation(cfg)
    dop = DistributedAdvectionOperation(cfg, rank=0, world_size=1)
    assert dop.layout.ghost_lo and dop.layout.ghost_hi
    integ = adv_lib.LowStorageRungeKuttaIntegrator(adv_lib.LSRK_5_4)
    dt = whole.time_step(0.5)
    assert dop.time_step(0.5) == dt
    uw, rw, kw = (whole.initialize_dof_vector() for _ in range(3))
    ud, rd, kd = (dop.initialize_dof_vector() for _ in range(3))
    whole.project_initial(uw)
    dop.project_initial(ud)
    for step in range(2):
        integ.perform_time_step(StageLoop(whole), step * dt, dt, uw, rw, kw)
        integ.perform_time_step(dop, step * dt, dt, ud, rd, kd)
    assert torch.equal(dop.layout.owned(ud), uw)
    assert abs(dop.l2_error(ud, 2 * dt)[0] - whole.l2_error(uw, 2 * dt)[0]) <= 1e-13


def test_slab_rejects_fused_loops(cuda, adv_lib):
    cfg = adv_lib.make_config(**CASES["curved-k4"])
    op = adv_lib.AdvectionOperation(cfg, slab=(1, 3))
    u, r, k = (op.initialize_dof_vector() for _ in range(3))
    with pytest.raises(adv_lib.AdvError):
        op.lsrk_steps(adv_lib.LSRK_5_4, 0.0, 1e-3, 1, u, r, k)
    with pytest.raises(adv_lib.AdvError):
        adv_lib.ImplicitSolver(op)
