"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE).

The oracle restates the reference miniapp's FP64 algorithm on the host (see
oracle.h for what is restated and for its parity status: unpinned against the
reference itself, pinned by self-made checks).  Only tests, the smoke check
and the CPU-baseline leg of the benchmark may import this module.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")


class OracleConfig(ctypes.Structure):
    _fields_ = [
        ("degree", ctypes.c_int32),
        ("n_cells", ctypes.c_int32 * 3),
        ("domain_lo", ctypes.c_double * 3),
        ("domain_hi", ctypes.c_double * 3),
        ("mesh_type", ctypes.c_int32),
        ("periodic", ctypes.c_int32),
        ("deformation", ctypes.c_double),
        ("velocity_type", ctypes.c_int32),
        ("initial_condition", ctypes.c_int32),
        ("velocity", ctypes.c_double * 3),
        ("velocity_period", ctypes.c_double),
        ("flux_alpha", ctypes.c_double),
        ("factor_skew", ctypes.c_double),
        ("diffusion", ctypes.c_double),
        ("penalty_factor", ctypes.c_double),
        ("boundary_value", ctypes.c_int32),
        ("reserved0", ctypes.c_int32),
        ("ic_params", ctypes.c_double * 8),
    ]


LSRK_3_3, LSRK_5_4, LSRK_7_4, LSRK_9_5 = 0, 1, 2, 3

_lib = None


def build(force=False):
    """Compile liboracle.so with the committed Makefile."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        D = ctypes.c_double
        dp = ctypes.POINTER(ctypes.c_double)
        L.oracle_create.argtypes = [ctypes.POINTER(OracleConfig), ctypes.POINTER(P)]
        L.oracle_destroy.argtypes = [P]
        L.oracle_n_dofs.argtypes = [P]
        L.oracle_n_dofs.restype = ctypes.c_int64
        L.oracle_n_cells.argtypes = [P]
        L.oracle_n_cells.restype = ctypes.c_int64
        L.oracle_set_num_threads.argtypes = [ctypes.c_int]
        L.oracle_get_max_threads.restype = ctypes.c_int
        L.oracle_tables.argtypes = [ctypes.c_int] + [dp] * 6
        for name in ("oracle_apply_unscaled", "oracle_apply", "oracle_apply_unscaled_dense"):
            getattr(L, name).argtypes = [P, dp, dp, D]
        for name in ("oracle_inverse_mass", "oracle_inverse_mass_dense"):
            getattr(L, name).argtypes = [P, dp, dp]
        L.oracle_perform_stage.argtypes = [P, D, D, D, dp, dp, dp, dp]
        L.oracle_lsrk_step.argtypes = [P, ctypes.c_int, D, D, dp, dp, dp]
        L.oracle_lsrk_coefficients.argtypes = [ctypes.c_int, dp, dp, ctypes.POINTER(ctypes.c_int)]
        L.oracle_project.argtypes = [P, D, dp]
        L.oracle_interpolate.argtypes = [P, D, dp]
        L.oracle_mass_energy.argtypes = [P, dp, dp]
        L.oracle_l2_error.argtypes = [P, dp, D, dp]
        L.oracle_time_step.argtypes = [P, D]
        L.oracle_time_step.restype = D
        L.oracle_min_vertex_distance.argtypes = [P]
        L.oracle_min_vertex_distance.restype = D
        L.oracle_support_points.argtypes = [P, dp]
        L.oracle_apply_mass.argtypes = [P, dp, dp]
        L.oracle_vmult.argtypes = [P, dp, dp, D, D]
        L.oracle_fdm_apply.argtypes = [P, dp, dp, dp, dp, dp, D]
        _lib = L
    return _lib


def _ptr(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_config(**kw):
    """Fill an OracleConfig from keyword arguments (same names as the fields)."""
    c = OracleConfig()
    c.degree = kw.get("degree", 3)
    for d, v in enumerate(kw.get("n_cells", (8, 8, 8))):
        c.n_cells[d] = v
    for d, v in enumerate(kw.get("domain_lo", (0.0, 0.0, 0.0))):
        c.domain_lo[d] = v
    for d, v in enumerate(kw.get("domain_hi", (1.0, 1.0, 1.0))):
        c.domain_hi[d] = v
    c.mesh_type = kw.get("mesh_type", 0)
    c.periodic = kw.get("periodic", 1)
    c.deformation = kw.get("deformation", 0.0)
    c.velocity_type = kw.get("velocity_type", 0)
    c.initial_condition = kw.get("initial_condition", 0)
    for d, v in enumerate(kw.get("velocity", (1.0, 0.15, -0.05))):
        c.velocity[d] = v
    c.velocity_period = kw.get("velocity_period", 1.0)
    c.flux_alpha = kw.get("flux_alpha", 1.0)
    c.factor_skew = kw.get("factor_skew", 0.0)
    c.diffusion = kw.get("diffusion", 0.0)
    c.penalty_factor = kw.get("penalty_factor", 1.0)
    c.boundary_value = kw.get("boundary_value", 1)
    for i, v in enumerate(kw.get("ic_params", ())):
        c.ic_params[i] = v
    return c


def tables(degree):
    n = degree + 1
    gl, gp, gw = np.zeros(n), np.zeros(n), np.zeros(n)
    S, D, Si = np.zeros((n, n)), np.zeros((n, n)), np.zeros((n, n))
    rc = lib().oracle_tables(degree, _ptr(gl), _ptr(gp), _ptr(gw), _ptr(S), _ptr(D), _ptr(Si))
    assert rc == 0
    return dict(gl=gl, gp=gp, gw=gw, S=S, D=D, Sinv=Si)


def lsrk_coefficients(scheme):
    a, b, n = np.zeros(16), np.zeros(16), ctypes.c_int()
    assert lib().oracle_lsrk_coefficients(scheme, _ptr(a), _ptr(b), ctypes.byref(n)) == 0
    return a[: n.value - 1].copy(), b[: n.value].copy()


def set_num_threads(n):
    lib().oracle_set_num_threads(int(n))


def max_threads():
    return lib().oracle_get_max_threads()


class Oracle:
    """FP64 CPU restatement of AdvectionOperation + LowStorageRungeKuttaIntegrator."""

    def __init__(self, config=None, **kw):
        self.config = config if config is not None else make_config(**kw)
        self._h = ctypes.c_void_p()
        rc = lib().oracle_create(ctypes.byref(self.config), ctypes.byref(self._h))
        if rc != 0:
            raise ValueError(f"oracle_create failed with {rc}")
        self.n_dofs = lib().oracle_n_dofs(self._h)
        self.n_cells = lib().oracle_n_cells(self._h)
        self.degree = self.config.degree

    def __del__(self):
        if getattr(self, "_h", None) and _lib is not None:
            _lib.oracle_destroy(self._h)
            self._h = None

    def zeros(self):
        return np.zeros(self.n_dofs)

    def apply(self, src, t=0.0):
        dst = self.zeros()
        assert lib().oracle_apply(self._h, _ptr(src), _ptr(dst), t) == 0
        return dst

    def apply_unscaled(self, src, t=0.0):
        dst = self.zeros()
        assert lib().oracle_apply_unscaled(self._h, _ptr(src), _ptr(dst), t) == 0
        return dst

    def apply_unscaled_dense(self, src, t=0.0):
        dst = self.zeros()
        assert lib().oracle_apply_unscaled_dense(self._h, _ptr(src), _ptr(dst), t) == 0
        return dst

    def inverse_mass(self, src):
        dst = self.zeros()
        assert lib().oracle_inverse_mass(self._h, _ptr(src), _ptr(dst)) == 0
        return dst

    def inverse_mass_dense(self, src):
        dst = self.zeros()
        assert lib().oracle_inverse_mass_dense(self._h, _ptr(src), _ptr(dst)) == 0
        return dst

    def perform_stage(self, t, b_dt, a_dt, r_in, k, u, r_out):
        rc = lib().oracle_perform_stage(self._h, t, b_dt, a_dt, _ptr(r_in), _ptr(k), _ptr(u), _ptr(r_out))
        assert rc == 0

    def lsrk_step(self, t, dt, u, r, k, scheme=LSRK_5_4):
        assert lib().oracle_lsrk_step(self._h, scheme, t, dt, _ptr(u), _ptr(r), _ptr(k)) == 0

    def project(self, t=0.0):
        dst = self.zeros()
        assert lib().oracle_project(self._h, t, _ptr(dst)) == 0
        return dst

    def interpolate(self, t=0.0):
        dst = self.zeros()
        assert lib().oracle_interpolate(self._h, t, _ptr(dst)) == 0
        return dst

    def mass_energy(self, u):
        out = np.zeros(3)
        assert lib().oracle_mass_energy(self._h, _ptr(u), _ptr(out)) == 0
        return out

    def l2_error(self, u, t):
        """(absolute L2 error, L2 norm of the exact solution)."""
        out = np.zeros(2)
        assert lib().oracle_l2_error(self._h, _ptr(u), t, _ptr(out)) == 0
        return out[0], out[1]

    def time_step(self, courant=0.5):
        return lib().oracle_time_step(self._h, courant)

    def min_vertex_distance(self):
        return lib().oracle_min_vertex_distance(self._h)

    def apply_mass(self, src):
        dst = self.zeros()
        assert lib().oracle_apply_mass(self._h, _ptr(src), _ptr(dst)) == 0
        return dst

    def vmult(self, src, mass_factor, t=0.0):
        """mass_factor M src - L(t) src (the implicit operator M/dt + A)."""
        dst = self.zeros()
        assert lib().oracle_vmult(self._h, _ptr(src), _ptr(dst), mass_factor, t) == 0
        return dst

    def fdm_apply(self, tables, src, mass_factor):
        """Block-Jacobi FDM preconditioner with tables = (lambda[2,n], V[2,n,n], VinvW[2,n,n]) complex."""
        lam, V, VW = (np.ascontiguousarray(np.stack([a.real, a.imag], axis=-1).reshape(-1)) for a in tables)
        dst = self.zeros()
        assert lib().oracle_fdm_apply(self._h, _ptr(lam), _ptr(V), _ptr(VW), _ptr(src), _ptr(dst), mass_factor) == 0
        return dst

    def support_points(self):
        xyz = np.zeros(self.n_dofs * 3)
        assert lib().oracle_support_points(self._h, _ptr(xyz)) == 0
        return xyz.reshape(-1, 3)
