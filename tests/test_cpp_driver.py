"""The C++ driver (the reference's main() against the C++ call surface in
include/advection_gb300.hpp) compiles, and on a GPU reproduces the 8^3 golden run."""
import os
import subprocess

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_driver_compiles(adv_lib):
    from advection_miniapp_gb300 import build
    assert os.path.exists(build.build_driver())


@pytest.mark.gpu
def test_driver_config1(cuda, adv_lib):
    from advection_miniapp_gb300 import build
    exe = build.build_driver()
    out = subprocess.run([exe, "3", "3", "200"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("Time")]
    final = float(lines[-1].split("error")[1].split()[0])
    gold = np.load(os.path.join(GOLDEN, "cartesian_k3_8.npz"))
    assert abs(final - float(gold["rel_l2"])) <= 1e-9 * float(gold["rel_l2"]), out.stdout
