"""Generate the golden fixtures of tests/golden from the CPU oracle.

The reference ships no outputs and cannot be built here (deal.II is absent),
so these fixtures freeze the oracle's results as regression pins for both the
oracle and the CUDA path:

* cartesian_k3_8.npz: the 8^3 affine periodic workload (degree 3, velocity
  (1, 0.15, -0.05), sine-product + Gaussian data, upwind, LSRK(5,4),
  Courant 0.5 / k^1.5), the projected initial vector, the final vector after
  200 steps, the relative L2 error and mass/energy at the end;
* operator_cases.npz: M^{-1} L applied to a seeded random vector on small
  meshes covering every face orientation, the periodic wrap, curved cells,
  Dirichlet faces, the skew-symmetric form and the rotating velocity.

Run: python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from oracle import oracle as O  # noqa: E402

OPERATOR_CASES = {
    "affine_k2_3x2x4": dict(degree=2, n_cells=(3, 2, 4)),
    "curved_k4_3": dict(degree=4, n_cells=(3, 3, 3), mesh_type=1, deformation=0.08),
    "dirichlet_skew_k3": dict(degree=3, n_cells=(2, 3, 2), periodic=0, factor_skew=0.5, initial_condition=2),
    "rotating_k3": dict(degree=3, n_cells=(3, 3, 2), periodic=0, velocity_type=1, velocity=(1.0, 1.0, 0.3),
                        velocity_period=0.5, initial_condition=1, ic_params=(0.3, 0.5, 0.5, 0.1),
                        boundary_value=0),
}


def config1():
    o = O.Oracle(degree=3, n_cells=(8, 8, 8))
    dt = o.time_step(0.5)
    u = o.project(0.0)
    u_init = u.copy()
    r, k = o.zeros(), o.zeros()
    t = 0.0
    for _ in range(200):
        o.lsrk_step(t, dt, u, r, k)
        t += dt
    err, nrm = o.l2_error(u, t)
    return dict(dt=dt, t_end=t, u_init=u_init, u_final=u, rel_l2=err / nrm,
                mass_energy=o.mass_energy(u))


def operator_cases():
    out = {}
    for name, cfg in OPERATOR_CASES.items():
        o = O.Oracle(**cfg)
        rng = np.random.default_rng(20240611)
        src = rng.standard_normal(o.n_dofs)
        out[name + "_src"] = src
        out[name + "_dst"] = o.apply(src, 0.25)
    return out


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "cartesian_k3_8.npz"), **config1())
    np.savez_compressed(os.path.join(HERE, "operator_cases.npz"), **operator_cases())
    print("written")
