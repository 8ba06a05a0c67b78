"""Return to the start, the reference's check of its variable-velocity and
implicit runs (advection_solver_variable.cc:1249-1252,
advection_solver_implicit.cc:1857-1860): the rotating field is scaled by
cos(pi t / T), so the flow reverses at T / 2 and every particle is back at
its start at T, and ||u(T) - u(0)||_inf measures the discretization error.

Pure advection (diffusion 0) of the degree-4 Gaussian blob of the
advection-diffusion workload on affine cells with zero Dirichlet inflow data,
LSRK(5,4) with T / dt a whole number of steps.  Measured on GB300 (relative
max norm): 8^3 5.96e-3, 12^3 1.22e-3, 16^3 3.11e-4, 24^3 3.73e-5 (order 5.2
between 16^3 and 24^3, the expected k + 1); half-way the blob has moved by
0.91 of its height; the FP32 operator gives the same errors to 1e-3
relative.
"""
import math

import pytest

pytestmark = pytest.mark.gpu


def _return_error(adv, torch, cells, precision):
    cfg = adv.workload_config("advection-diffusion-k5-32", precision=precision, diffusion=0.0, degree=4,
                              n_cells=(cells,) * 3)
    op = adv.AdvectionOperation(cfg)
    period = cfg.velocity_period
    n = math.ceil(period / op.time_step(0.5))
    dt = period / n
    u0 = op.initialize_dof_vector()
    op.project_initial(u0)
    u, r, k = u0.clone(), op.initialize_dof_vector(), op.initialize_dof_vector()
    half = u0.clone()
    op.lsrk_steps(adv.LSRK_5_4, 0.0, dt, n // 2, half, r, k)
    op.lsrk_steps(adv.LSRK_5_4, 0.0, dt, n, u, r, k)
    torch.cuda.synchronize()
    scale = u0.abs().max()
    out = (((u - u0).abs().max() / scale).item(), ((half - u0).abs().max() / scale).item())
    op.close()
    return out


def test_return_to_start_converges(cuda, adv_lib):
    torch, adv = cuda, adv_lib
    e8, h8 = _return_error(adv, torch, 8, adv.PRECISION_FP64)
    e16, h16 = _return_error(adv, torch, 16, adv.PRECISION_FP64)
    # the blob has left its start half-way and is back at T
    assert h8 > 0.5 and h16 > 0.5
    assert e16 < 5e-4
    # order > 3.6 between 8^3 and 16^3 (measured 4.3; k + 1 = 5 asymptotically)
    assert e16 < 0.08 * e8, (e8, e16)


def test_return_to_start_fp32_operator_matches_fp64(cuda, adv_lib):
    torch, adv = cuda, adv_lib
    e64, _ = _return_error(adv, torch, 16, adv.PRECISION_FP64)
    e32, _ = _return_error(adv, torch, 16, adv.PRECISION_FP32_OPERATOR)
    assert e32 <= 1.05 * e64 and e64 <= 1.05 * e32, (e64, e32)
