"""The C-ABI library: builds, loads, exports every declared symbol, validates
arguments on the host (no GPU needed), and its struct layout matches the C
header."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "advection_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(adv_[a-z0-9_]+)\s*\(", text)))


def test_exports_every_declared_symbol(adv_lib):
    from advection_miniapp_gb300 import _lib
    L = _lib.load()
    names = declared_functions()
    assert len(names) >= 20
    for name in names:
        assert hasattr(L, name), name
    # and the Python binding covers all of them
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_struct_layout_matches_header(adv_lib, tmp_path):
    from advection_miniapp_gb300 import AdvConfig
    src = tmp_path / "layout.c"
    fields = [f for f, _ in AdvConfig._fields_]
    body = "\n".join(f'  printf("{f} %zu\\n", offsetof(adv_config, {f}));' for f in fields)
    src.write_text(f'#include <stdio.h>\n#include <stddef.h>\n#include "advection_gb300.h"\n'
                   f'int main(void) {{\n{body}\n  printf("sizeof %zu\\n", sizeof(adv_config));\n  return 0;\n}}\n')
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    for f in fields:
        assert int(out[f]) == getattr(AdvConfig, f).offset, f
    assert int(out["sizeof"]) == ctypes.sizeof(AdvConfig)


def test_config_prefix_matches_oracle(adv_lib, oracle_mod):
    from advection_miniapp_gb300 import AdvConfig
    for name, _ in oracle_mod.OracleConfig._fields_:
        assert getattr(AdvConfig, name).offset == getattr(oracle_mod.OracleConfig, name).offset, name


def test_default_config(adv_lib):
    c = adv_lib.make_config()
    assert c.degree == 3 and list(c.n_cells) == [8, 8, 8]
    assert list(c.velocity) == [1.0, 0.15, -0.05]
    assert c.flux_alpha == 1.0 and c.periodic == 1 and c.precision == 0


@pytest.mark.parametrize("bad", [
    dict(degree=0), dict(degree=7), dict(n_cells=(0, 4, 4)), dict(domain_hi=(0.0, 1.0, 1.0)),
    dict(mesh_type=5), dict(mesh_type=1, deformation=0.5), dict(velocity_type=3),
    dict(velocity_type=1, velocity_period=0.0), dict(precision=7), dict(initial_condition=9),
    dict(initial_condition=1, ic_params=(0.5, 0.5, 0.5, 0.0)), dict(flux_alpha=2.0),
    dict(fused_form=9), dict(diffusion=-1.0), dict(diffusion=1e-3, mesh_type=1, deformation=0.05),
    dict(diffusion=1e-3, penalty_factor=0.0),
])
def test_invalid_configs_rejected_on_host(adv_lib, bad):
    from advection_miniapp_gb300 import _lib
    L = _lib.load()
    c = adv_lib.make_config(**bad)
    h = ctypes.c_void_p()
    rc = L.adv_create(ctypes.byref(c), ctypes.byref(h))
    assert rc == 1
    assert h.value is None
    assert len(L.adv_last_error()) > 0


def test_null_arguments(adv_lib):
    from advection_miniapp_gb300 import _lib
    L = _lib.load()
    assert L.adv_create(None, None) == 1
    assert L.adv_apply(None, None, None, 0.0, None) == 1
    assert L.adv_lsrk_steps(None, 1, 0.0, 0.1, 1, None, None, None, None) == 1
    assert L.adv_lsrk_steps_host(None, 1, 0.0, 0.1, 1, None, None, None, None, None) == 1
    assert L.adv_destroy(None) == 0


def test_lsrk_coefficients_match_oracle(adv_lib, oracle_mod):
    for scheme in range(4):
        a, b = adv_lib.lsrk_coefficients(scheme)
        ao, bo = oracle_mod.lsrk_coefficients(scheme)
        np.testing.assert_array_equal(a, ao)
        np.testing.assert_array_equal(b, bo)
    from advection_miniapp_gb300 import _lib
    assert _lib.load().adv_lsrk_coefficients(9, None, None, None) == 1


def test_host_only_entry_points_reject_bad_input(adv_lib):
    """Slab layouts and the serving loop check their arguments before any
    device work."""
    from advection_miniapp_gb300 import _lib
    L = _lib.load()
    c = adv_lib.make_config(n_cells=(4, 4, 6))
    out = (ctypes.c_int64 * 10)()
    for zb, ze in ((-1, 3), (2, 2), (3, 7)):
        assert L.adv_slab_layout(ctypes.byref(c), zb, ze, out) == 1
    assert L.adv_slab_layout(ctypes.byref(c), 0, 6, out) == 0 and out[8] == 8  # periodic: two ghost layers
    s = ctypes.c_void_p()
    assert L.adv_server_create(0, 8, 16, 0, ctypes.byref(s)) == 1
    assert L.adv_server_create(1 << 30, 0, 16, 0, ctypes.byref(s)) == 1
    assert L.adv_server_create(1 << 30, 8, 0, 0, ctypes.byref(s)) == 1
    assert L.adv_server_set_policy(None, 0) == 1
    assert L.adv_write_vtu_host(ctypes.byref(adv_lib.make_config(degree=0)), None, 0.0, b"x.vtu") == 1
