"""The oracle reproduces its committed golden fixtures (tests/golden/gen_golden.py)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_config1_golden(oracle_mod):
    g = np.load(os.path.join(GOLDEN, "cartesian_k3_8.npz"))
    o = oracle_mod.Oracle(degree=3, n_cells=(8, 8, 8))
    assert abs(o.time_step(0.5) - float(g["dt"])) < 1e-16
    u = o.project(0.0)
    np.testing.assert_allclose(u, g["u_init"], rtol=0, atol=1e-14)
    r, k = o.zeros(), o.zeros()
    dt, t = float(g["dt"]), 0.0
    for _ in range(200):
        o.lsrk_step(t, dt, u, r, k)
        t += dt
    scale = np.abs(g["u_final"]).max()
    assert np.abs(u - g["u_final"]).max() <= 1e-12 * scale
    err, nrm = o.l2_error(u, t)
    assert abs(err / nrm - float(g["rel_l2"])) <= 1e-10 * float(g["rel_l2"])


def test_operator_golden(oracle_mod):
    import sys
    sys.path.insert(0, GOLDEN)
    from gen_golden import OPERATOR_CASES
    g = np.load(os.path.join(GOLDEN, "operator_cases.npz"))
    for name, cfg in OPERATOR_CASES.items():
        o = oracle_mod.Oracle(**cfg)
        dst = o.apply(g[name + "_src"], 0.25)
        ref = g[name + "_dst"]
        assert np.abs(dst - ref).max() <= 1e-12 * np.abs(ref).max(), name
