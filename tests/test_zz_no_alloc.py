"""adv_perform_stage_noalloc: the stage entry point for callers that must not
allocate device memory mid-solve (memory-budgeted serving, latency-critical
loops, memory owned by another allocator).  It stages an output that aliases
r_in in a static device array instead of a lazily allocated handle vector.

Called through the C ABI (ctypes) and checked against adv_perform_stage on
the reference's stage patterns, two calls in a row.  Runs alone in a fresh
process as well as after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # the FP64 parity bar of the other GPU tests


def _setup(adv_lib, torch, **cfg):
    from advection_miniapp_gb300 import _lib
    L = _lib.load()
    c = adv_lib.make_config(**cfg)
    h = ctypes.c_void_p()
    assert L.adv_create(ctypes.byref(c), ctypes.byref(h)) == 0, L.adv_last_error()
    n = ctypes.c_int64()
    assert L.adv_n_dofs(h, ctypes.byref(n)) == 0
    return L, h, n.value


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream(torch):
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def rel(a, b):
    a, b = a.cpu().numpy(), b.cpu().numpy()
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_noalloc_stage_matches_perform_stage(cuda, adv_lib):
    torch = cuda
    L, h, n = _setup(adv_lib, torch, degree=4, n_cells=(6, 5, 4), mesh_type=1, deformation=0.08)
    try:
        assert n <= 1 << 21
        rng = np.random.default_rng(42)
        u0 = torch.from_numpy(rng.standard_normal(n)).cuda()
        r0 = torch.from_numpy(rng.standard_normal(n)).cuda()
        # reference path (adv_perform_stage) and the allocation-free path on copies
        u1, r1, k1 = u0.clone(), r0.clone(), torch.zeros_like(u0)
        u2, r2, k2 = u0.clone(), r0.clone(), torch.zeros_like(u0)
        s = _stream(torch)
        b, a, t = 0.013, 0.021, 0.3
        # call 1: first-stage pattern perform_stage(t, b, a, u, r, u, r): r_in aliases u
        assert L.adv_perform_stage(h, t, b, a, _p(u1), _p(r1), _p(u1), _p(r1), s) == 0
        assert L.adv_perform_stage_noalloc(h, t, b, a, _p(u2), _p(r2), _p(u2), _p(r2), s) == 0, \
            L.adv_last_error()
        torch.cuda.synchronize()
        assert rel(u2, u1) <= TOL and rel(r2, r1) <= TOL
        # call 2, right after: later-stage pattern perform_stage(t, b, a, r, k, u, r): r_out aliases r_in
        assert L.adv_perform_stage(h, t + 0.01, b, a, _p(r1), _p(k1), _p(u1), _p(r1), s) == 0
        assert L.adv_perform_stage_noalloc(h, t + 0.01, b, a, _p(r2), _p(k2), _p(u2), _p(r2), s) == 0, \
            L.adv_last_error()
        torch.cuda.synchronize()
        assert rel(u2, u1) <= TOL and rel(r2, r1) <= TOL
    finally:
        L.adv_destroy(h)


def test_noalloc_stage_allocates_nothing(cuda, adv_lib):
    """Free device memory is the same before the first call and after the
    calls: the static array is committed when the handle is created, not by
    a stage call."""
    torch = cuda
    L, h, n = _setup(adv_lib, torch, degree=3, n_cells=(8, 8, 8))
    try:
        u = torch.from_numpy(np.random.default_rng(1).standard_normal(n)).cuda()
        r, k, v, w = (torch.zeros_like(u) for _ in range(4))
        s = _stream(torch)
        # a stage with no aliasing (which stages nothing) loads the stage
        # kernel's code on the device, which the driver may place in newly
        # committed memory
        assert L.adv_perform_stage(h, 0.0, 0.01, 0.02, _p(v), _p(k), _p(u), _p(w), s) == 0
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        for _ in range(2):
            assert L.adv_perform_stage_noalloc(h, 0.0, 0.01, 0.02, _p(u), _p(r), _p(u), _p(r), s) == 0
            assert L.adv_perform_stage_noalloc(h, 0.0, 0.01, 0.02, _p(r), _p(k), _p(u), _p(r), s) == 0
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_before
    finally:
        L.adv_destroy(h)


def test_noalloc_stage_is_timed_like_the_other_entry_points(cuda, adv_lib):
    torch = cuda
    L, h, n = _setup(adv_lib, torch, degree=2, n_cells=(4, 4, 4))
    try:
        u = torch.from_numpy(np.random.default_rng(2).standard_normal(n)).cuda()
        r, k = torch.zeros_like(u), torch.zeros_like(u)
        s = _stream(torch)
        assert L.adv_set_timing(h, 1) == 0
        for _ in range(3):
            assert L.adv_perform_stage_noalloc(h, 0.0, 0.01, 0.02, _p(u), _p(r), _p(u), _p(r), s) == 0
        sec, calls = ctypes.c_double(), ctypes.c_int64()
        assert L.adv_timing(h, ctypes.byref(sec), ctypes.byref(calls)) == 0
        assert calls.value == 3 and sec.value > 0.0
    finally:
        L.adv_destroy(h)


def test_noalloc_stage_rejects_meshes_above_the_limit(cuda, adv_lib):
    torch = cuda
    L, h, n = _setup(adv_lib, torch, degree=3, n_cells=(33, 33, 33))
    try:
        assert n > 1 << 21
        buf = torch.zeros(8, dtype=torch.float64, device="cuda")
        rc = L.adv_perform_stage_noalloc(h, 0.0, 0.01, 0.0, _p(buf), _p(buf), _p(buf), _p(buf), _stream(torch))
        assert rc == 1
        assert b"ADV_NOALLOC_MAX_DOFS" in L.adv_last_error()
    finally:
        L.adv_destroy(h)
