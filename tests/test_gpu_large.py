"""Maximum sizes: a mesh with more than 2^31 DoFs (272^3 affine periodic
cells of degree 4, 2,515,456,000 DoFs; about 110 GB of device memory with the
step loop's face traces).  Every index into the vectors, the traces and the
face data must be 64-bit: an overflow anywhere shows as an O(1) error."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_more_than_2_31_dofs(cuda, adv_lib):
    torch = cuda
    free, total = torch.cuda.mem_get_info()
    if free < 130 * 2 ** 30:
        pytest.skip("needs about 110 GB of free device memory")
    op = adv_lib.AdvectionOperation(degree=4, n_cells=(272, 272, 272), velocity=(1.0, 0.15, -0.05))
    assert op.n_dofs == 272 ** 3 * 125 > 2 ** 31
    u = op.initialize_dof_vector()
    op.project_initial(u)
    e0, n0 = op.l2_error(u, 0.0)
    m0 = op.compute_mass_and_energy(u)
    r, k = op.initialize_dof_vector(), op.initialize_dof_vector()
    dt = op.time_step(0.5)
    op.lsrk_steps(adv_lib.LSRK_5_4, 0.0, dt, 2, u, r, k)
    e, nrm = op.l2_error(u, 2 * dt)
    m = op.compute_mass_and_energy(u)
    # the projection error is 1.3e-12; the steps add about 6e-7 per unit time
    # at any resolution (the Gaussian part of the data is not periodic: its
    # derivative jumps by 4e-4 across the domain boundary), 3e-10 here; an
    # index overflow anywhere would show as an O(1) error
    assert e0 / n0 < 1e-11 and e / nrm < 1e-9, (e / nrm, e0 / n0)
    assert abs(m[0] - m0[0]) <= 1e-12 * abs(m0[1]) ** 0.5
    assert torch.isfinite(u[-125 * 4096:]).all()
    del u, r, k
    torch.cuda.empty_cache()
