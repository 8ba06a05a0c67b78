"""adv_lsrk_steps_host: time steps on a solution in host memory.

The copies run in chunks of z layers, overlapped with the change to the
Gauss basis (collocation form) or the first stage (nodal form) and with the
last stage, which then launch chunk by chunk.  Every cell gets the same
arithmetic as in adv_lsrk_steps, so the results must agree bit for bit, for
every form
(collocation with and without traces, nodal, FP32 increments), on periodic
and Dirichlet meshes, and for chunk counts from one to eight (including
chunks of a single layer whose lower and upper neighbour layers coincide).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    # 13.8 MB of DoFs: 6 chunks of 4 layers
    "deformed-k4-24": dict(degree=4, n_cells=(24, 24, 24), mesh_type=1, deformation=0.08,
                           velocity=(1.0, 0.15, -0.05)),
    # 2 chunks over 3 layers (1 + 2)
    "flat-k4-3-layers": dict(degree=4, n_cells=(40, 40, 3), velocity=(0.4, -0.3, 1.0)),
    # 2 chunks of one layer: each chunk's lower and upper neighbour is the other
    "two-layers-periodic": dict(degree=4, n_cells=(64, 64, 2), velocity=(0.2, 0.1, 1.0)),
    # 8 chunks (the cap) of 8 layers
    "affine-k3-64": dict(degree=3, n_cells=(32, 32, 64), velocity=(0.3, 0.2, 1.0)),
    # one chunk
    "small-k2": dict(degree=2, n_cells=(3, 4, 5)),
    "dirichlet-exact-k3": dict(degree=3, n_cells=(24, 24, 20), periodic=0, initial_condition=2,
                               boundary_value=1, mesh_type=1, deformation=0.05),
    "rotating-k3": dict(degree=3, n_cells=(24, 24, 24), periodic=0, velocity_type=1, velocity=(1.0, 1.0, 0.3),
                        velocity_period=0.5, initial_condition=1, ic_params=(0.3, 0.5, 0.5, 0.1),
                        boundary_value=0),
    "sipg-k3": dict(degree=3, n_cells=(20, 20, 24), diffusion=1e-2),
    # zero Dirichlet data, constant velocity: the FP32 increment form with boundary faces
    "dirichlet-zero-k4": dict(degree=4, n_cells=(16, 16, 12), periodic=0, boundary_value=0, initial_condition=1,
                              ic_params=(0.5, 0.5, 0.5, 0.15), mesh_type=1, deformation=0.05),
    # an odd number of DoFs (105 cells of 125): registers and cells off 16 bytes
    "odd-dofs-k4": dict(degree=4, n_cells=(5, 3, 7), mesh_type=1, deformation=0.05),
}


def _run_both(torch, adv, cfg, precision, n_steps, scheme, form=None):
    kw = dict(cfg, precision=precision)
    if form is not None:
        kw["fused_form"] = form
    op = adv.AdvectionOperation(**kw)
    dt = op.time_step(0.3)
    u0 = op.initialize_dof_vector()
    op.project_initial(u0)
    # reference: the device step loop
    u, r, k = u0.clone(), op.initialize_dof_vector(), op.initialize_dof_vector()
    op.lsrk_steps(scheme, 0.1, dt, n_steps, u, r, k)
    # host path, with a device vector holding something else beforehand
    host = torch.empty(op.n_dofs, dtype=torch.float64, pin_memory=True)
    host.copy_(u0.cpu())
    ud, rd, kd = op.initialize_dof_vector(), op.initialize_dof_vector(), op.initialize_dof_vector()
    ud.fill_(7.0)
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        op.lsrk_steps_host(scheme, 0.1, dt, n_steps, host, ud, rd, kd, stream=s)
    s.synchronize()
    ref = u.cpu().numpy()
    out = host.numpy().copy()
    dev = ud.cpu().numpy()
    op.close()
    return ref, out, dev


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_host_steps_equal_device_steps(cuda, adv_lib, case, precision):
    torch, adv = cuda, adv_lib
    ref, out, dev = _run_both(torch, adv, CASES[case], precision, 2, adv.LSRK_5_4)
    assert np.isfinite(ref).all()
    assert np.array_equal(out, ref)
    assert np.array_equal(dev, ref)


@pytest.mark.parametrize("form", [1, 2, 3])
@pytest.mark.parametrize("n_steps", [1, 3])
@pytest.mark.parametrize("precision", [0, 2])
def test_host_steps_every_form(cuda, adv_lib, form, n_steps, precision):
    torch, adv = cuda, adv_lib
    ref, out, dev = _run_both(torch, adv, CASES["deformed-k4-24"], precision, n_steps, adv.LSRK_3_3, form=form)
    assert np.array_equal(out, ref) and np.array_equal(dev, ref)


@pytest.mark.parametrize("interval", [1, 2, 3])
def test_host_steps_increment_blocks(cuda, adv_lib, interval):
    """FP32 increments over several anchor blocks (face traces of each later
    anchor from a traces-only launch) through the host path."""
    torch, adv = cuda, adv_lib
    cfg = dict(CASES["deformed-k4-24"], anchor_interval=interval)
    ref, out, dev = _run_both(torch, adv, cfg, 2, 7, adv.LSRK_5_4)
    assert np.array_equal(out, ref) and np.array_equal(dev, ref)


def test_host_steps_pageable_host_memory(cuda, adv_lib):
    """Host memory that is not page-locked: the copies cannot overlap, the
    results are the same."""
    torch, adv = cuda, adv_lib
    op = adv.AdvectionOperation(**CASES["deformed-k4-24"])
    dt = op.time_step(0.5)
    u0 = op.initialize_dof_vector()
    op.project_initial(u0)
    u, r, k = u0.clone(), op.initialize_dof_vector(), op.initialize_dof_vector()
    op.lsrk_steps(adv.LSRK_5_4, 0.0, dt, 2, u, r, k)
    host = u0.cpu().clone()
    assert not host.is_pinned()
    ud, rd, kd = op.initialize_dof_vector(), op.initialize_dof_vector(), op.initialize_dof_vector()
    torch.cuda.synchronize()
    op.lsrk_steps_host(adv.LSRK_5_4, 0.0, dt, 2, host, ud, rd, kd)
    torch.cuda.synchronize()
    assert np.array_equal(host.numpy(), u.cpu().numpy())
    op.close()


def test_host_steps_zero_steps_copies_in(cuda, adv_lib):
    torch, adv = cuda, adv_lib
    op = adv.AdvectionOperation(**CASES["small-k2"])
    u0 = op.initialize_dof_vector()
    op.project_initial(u0)
    host = u0.cpu().pin_memory()
    ud, r, k = op.initialize_dof_vector(), op.initialize_dof_vector(), op.initialize_dof_vector()
    op.lsrk_steps_host(adv.LSRK_5_4, 0.0, 1e-3, 0, host, ud, r, k)
    torch.cuda.synchronize()
    assert torch.equal(ud, u0)
    assert torch.equal(host, u0.cpu())
    op.close()


def test_host_steps_back_to_back_calls(cuda, adv_lib):
    """Consecutive calls on one stream (the next call's copy in waits for the
    previous call's copy out) equal one call of all the steps."""
    torch, adv = cuda, adv_lib
    op = adv.AdvectionOperation(**CASES["deformed-k4-24"])
    dt = op.time_step(0.5)
    u0 = op.initialize_dof_vector()
    op.project_initial(u0)
    u, r, k = u0.clone(), op.initialize_dof_vector(), op.initialize_dof_vector()
    op.lsrk_steps(adv.LSRK_5_4, 0.0, dt, 4, u, r, k)
    host = u0.cpu().pin_memory()
    ud, rd, kd = op.initialize_dof_vector(), op.initialize_dof_vector(), op.initialize_dof_vector()
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        for i in range(4):
            op.lsrk_steps_host(adv.LSRK_5_4, i * dt, dt, 1, host, ud, rd, kd, stream=s)
    s.synchronize()
    # per-step calls change the basis back and forth between steps: equal to
    # round-off, not bit for bit
    ref = u.cpu().numpy()
    assert np.abs(host.numpy() - ref).max() <= 1e-13 * np.abs(ref).max()
    op.close()


def test_host_steps_rejects_bad_arguments(cuda, adv_lib):
    torch, adv = cuda, adv_lib
    op = adv.AdvectionOperation(**CASES["small-k2"])
    u, r, k = op.initialize_dof_vector(), op.initialize_dof_vector(), op.initialize_dof_vector()
    with pytest.raises(ValueError):
        op.lsrk_steps_host(adv.LSRK_5_4, 0.0, 1e-3, 1, u, u, r, k)  # a device tensor as host data
    with pytest.raises(ValueError):
        op.lsrk_steps_host(adv.LSRK_5_4, 0.0, 1e-3, 1, torch.zeros(3, dtype=torch.float64), u, r, k)
    host = torch.zeros(op.n_dofs, dtype=torch.float64)
    with pytest.raises(RuntimeError):
        op.lsrk_steps_host(adv.LSRK_5_4, 0.0, 1e-3, 1, host, u, u, k)  # aliasing
    op.close()
