"""GB300-native matrix-free DG advection operator with the reference's call surface.

`AdvectionOperation` and `LowStorageRungeKuttaIntegrator` mirror the classes
of the reference miniapp (advection_solver.cc:329-431 and 822-944) over the C
ABI of libadvection_gb300.so.  Vectors are CUDA float64 torch tensors of
`n_dofs` entries (torch is used for device memory and streams only); every
computation runs in the library's sm_103a kernels.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import (AdvConfig, AdvError, BOUNDARY_EXACT, BOUNDARY_ZERO, FORM_AUTO, FORM_COLLOCATION, FORM_COLLOCATION_NO_TRACES,
                   FORM_NODAL,
                   IC_BLOB, IC_SINE_GAUSS,
                   IC_WAVE, LSRK_3_3, LSRK_5_4, LSRK_7_4, LSRK_9_5, MESH_CARTESIAN, MESH_DEFORMED,
                   PRECISION_FP32_INCREMENT, PRECISION_FP32_OPERATOR, PRECISION_FP64, VELOCITY_CONSTANT,
                   VELOCITY_ROTATING)

__all__ = [
    "AdvConfig", "AdvError", "AdvectionOperation", "ImplicitSolver", "LowStorageRungeKuttaIntegrator", "make_config",
    "workload_config", "lsrk_coefficients", "measure_fma_peak",
]


def make_config(**kw):
    """adv_config from keyword arguments named like its fields (defaults: adv_config_default)."""
    lib = _lib.load()
    c = AdvConfig()
    lib.adv_config_default(ctypes.byref(c))
    for key, val in kw.items():
        if not hasattr(c, key):
            raise KeyError(f"unknown adv_config field {key!r}")
        field = getattr(c, key)
        if isinstance(field, ctypes.Array):
            for i, v in enumerate(val):
                field[i] = v
        else:
            setattr(c, key, val)
    return c


def workload_config(name, precision=PRECISION_FP64, **overrides):
    """Configurations of the benchmark workloads.

    * ``"cartesian-k3-8"``: unit cube, 8^3 affine periodic cells, degree 3,
      velocity (1, 0.15, -0.05), sine-product + Gaussian initial data, upwind.
    * ``"deformed-k4-64"``: the same PDE on 64^3 cells of the sine-deformed
      cube (amplitude 0.08), degree 4, 32,768,000 DoFs.
    * ``"deformed-k4-32"``: 32^3 deformed cells, degree 4, 4,096,000 DoFs (the
      implicit BDF2 workload).
    * ``"advection-diffusion-k5-32"``: 32^3 affine cells, degree 5, rotating
      field times cos(pi t / 0.5), SIPG diffusion 1e-3 with penalty
      (k+1)^2/h, Dirichlet-zero boundaries, Gaussian blob of width 0.1 at
      (0.3, 0.5, 0.5).
    """
    base = dict(velocity=(1.0, 0.15, -0.05), flux_alpha=1.0, initial_condition=IC_SINE_GAUSS,
                periodic=1, precision=precision)
    if name == "cartesian-k3-8":
        base.update(degree=3, n_cells=(8, 8, 8), mesh_type=MESH_CARTESIAN)
    elif name == "deformed-k4-64":
        base.update(degree=4, n_cells=(64, 64, 64), mesh_type=MESH_DEFORMED, deformation=0.08)
    elif name == "deformed-k4-32":
        base.update(degree=4, n_cells=(32, 32, 32), mesh_type=MESH_DEFORMED, deformation=0.08)
    elif name == "advection-diffusion-k5-32":
        base.update(degree=5, n_cells=(32, 32, 32), mesh_type=MESH_CARTESIAN, periodic=0,
                    velocity_type=VELOCITY_ROTATING, velocity=(1.0, 1.0, 0.3), velocity_period=0.5,
                    diffusion=1e-3, penalty_factor=1.0, initial_condition=IC_BLOB,
                    ic_params=(0.3, 0.5, 0.5, 0.1), boundary_value=BOUNDARY_ZERO)
    else:
        raise KeyError(name)
    base.update(overrides)
    return make_config(**base)


def lsrk_coefficients(scheme):
    """(a, b) of a low-storage Runge-Kutta scheme (a has n_stages - 1 entries)."""
    a = (ctypes.c_double * 16)()
    b = (ctypes.c_double * 16)()
    n = ctypes.c_int()
    _lib.check(_lib.load().adv_lsrk_coefficients(scheme, a, b, ctypes.byref(n)), "adv_lsrk_coefficients")
    return np.array(a[: n.value - 1]), np.array(b[: n.value])


def write_vtu_host(config, values, time, path):
    """VTU output of host values (numpy, n_dofs of the whole mesh); no GPU needed."""
    v = np.ascontiguousarray(values, dtype=np.float64)
    _lib.check(_lib.load().adv_write_vtu_host(ctypes.byref(config), v.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                              float(time), str(path).encode()), "adv_write_vtu_host")


def _stream_handle(stream):
    import torch
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def measure_fma_peak(precision=PRECISION_FP64, stream=None):
    """Measured FMA throughput (TFLOP/s, FMA = 2 flops) of the current GPU."""
    out = ctypes.c_double()
    _lib.check(_lib.load().adv_measure_fma_peak(precision, ctypes.byref(out), _stream_handle(stream)),
               "adv_measure_fma_peak")
    return out.value


class AdvectionOperation:
    """GB300 counterpart of the reference's AdvectionOperation<dim, fe_degree>.

    reinit (advection_solver.cc:435-465) happens at construction from an
    adv_config (or keyword arguments for make_config).  With slab=(z_begin,
    z_end) the operator covers those global z layers of the mesh plus ghost
    layers (adv_create_slab); the distributed module drives such slabs.
    """

    def __init__(self, config=None, slab=None, **kw):
        self._lib = _lib.load()
        self.config = config if config is not None else make_config(**kw)
        self._h = ctypes.c_void_p()
        self.slab = tuple(slab) if slab is not None else None
        if self.slab is None:
            _lib.check(self._lib.adv_create(ctypes.byref(self.config), ctypes.byref(self._h)), "adv_create")
        else:
            _lib.check(self._lib.adv_create_slab(ctypes.byref(self.config), int(self.slab[0]), int(self.slab[1]),
                                                 ctypes.byref(self._h)), "adv_create_slab")
        n = ctypes.c_int64()
        _lib.check(self._lib.adv_n_dofs(self._h, ctypes.byref(n)), "adv_n_dofs")
        self.n_dofs = n.value
        _lib.check(self._lib.adv_n_cells(self._h, ctypes.byref(n)), "adv_n_cells")
        self.n_cells = n.value
        self.degree = self.config.degree

    def close(self):
        if getattr(self, "_h", None):
            self._lib.adv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- vectors -----------------------------------------------------------
    def _ptr(self, vec):
        import torch
        if not (isinstance(vec, torch.Tensor) and vec.is_cuda and vec.dtype == torch.float64
                and vec.is_contiguous() and vec.numel() == self.n_dofs):
            raise ValueError(f"expected a contiguous CUDA float64 tensor of {self.n_dofs} entries")
        return ctypes.c_void_p(vec.data_ptr())

    def initialize_dof_vector(self):
        """A zeroed vector of the operator's layout (advection_solver.cc:343-347)."""
        import torch
        return torch.zeros(self.n_dofs, dtype=torch.float64, device="cuda")

    # -- the reference's member functions ----------------------------------
    def apply(self, src, dst, current_time, stream=None):
        """dst = M^{-1} L(t) src (advection_solver.cc:661-691)."""
        _lib.check(self._lib.adv_apply(self._h, self._ptr(src), self._ptr(dst), float(current_time),
                                       _stream_handle(stream)), "adv_apply")

    def perform_stage(self, current_time, factor_solution, factor_ai, current_ri, vec_ki, solution,
                      next_ri, stream=None):
        """One LSRK stage (advection_solver.cc:695-756); vec_ki is scratch."""
        _lib.check(self._lib.adv_perform_stage(
            self._h, float(current_time), float(factor_solution), float(factor_ai),
            self._ptr(current_ri), self._ptr(vec_ki), self._ptr(solution),
            self._ptr(next_ri) if next_ri is not None else None, _stream_handle(stream)),
            "adv_perform_stage")

    def project_initial(self, dst, time=0.0, stream=None):
        """L2 projection of the exact solution at `time` (advection_solver.cc:760-784)."""
        _lib.check(self._lib.adv_project(self._h, float(time), self._ptr(dst), _stream_handle(stream)),
                   "adv_project")

    def compute_mass_and_energy(self, vec, stream=None):
        """[int u, int u^2, int |grad u|^2] (advection_solver.cc:787-818)."""
        out = (ctypes.c_double * 3)()
        _lib.check(self._lib.adv_mass_energy(self._h, self._ptr(vec), out, _stream_handle(stream)),
                   "adv_mass_energy")
        return np.array(out[:])

    def l2_error(self, vec, time, stream=None):
        """(||u_h - u(t)|| with QGauss(k+2), ||u(t)|| with QGauss(k+1)) as in output_results."""
        out = (ctypes.c_double * 2)()
        _lib.check(self._lib.adv_l2_error(self._h, self._ptr(vec), float(time), out, _stream_handle(stream)),
                   "adv_l2_error")
        return out[0], out[1]

    def time_step(self, courant=0.5):
        """courant * h_min / |a| / k^1.5 (advection_solver.cc:1155-1165, before rounding)."""
        dt = ctypes.c_double()
        _lib.check(self._lib.adv_time_step(self._h, float(courant), ctypes.byref(dt)), "adv_time_step")
        return dt.value

    def launch_count(self):
        n = ctypes.c_int64()
        _lib.check(self._lib.adv_launch_count(self._h, ctypes.byref(n)), "adv_launch_count")
        return n.value

    def device_bytes(self):
        n = ctypes.c_int64()
        _lib.check(self._lib.adv_device_bytes(self._h, ctypes.byref(n)), "adv_device_bytes")
        return n.value

    # -- implicit operator (advection_solver_implicit.cc) ---------------------
    def vmult(self, src, dst, mass_factor, time=0.0, stream=None):
        """dst = mass_factor M src - L(t) src (the reference's vmult = M/dt + A)."""
        _lib.check(self._lib.adv_vmult(self._h, self._ptr(src), self._ptr(dst), float(mass_factor), float(time),
                                       _stream_handle(stream)), "adv_vmult")

    def apply_mass(self, src, dst, stream=None):
        _lib.check(self._lib.adv_apply_mass(self._h, self._ptr(src), self._ptr(dst), _stream_handle(stream)),
                   "adv_apply_mass")

    # -- timing (computing_times, advection_solver.cc:349-372) -------------
    def set_timing(self, enable=True):
        _lib.check(self._lib.adv_set_timing(self._h, 1 if enable else 0), "adv_set_timing")

    def timing(self):
        """(device seconds, calls) accumulated by the timed calls so far."""
        sec, calls = ctypes.c_double(), ctypes.c_int64()
        _lib.check(self._lib.adv_timing(self._h, ctypes.byref(sec), ctypes.byref(calls)), "adv_timing")
        return sec.value, calls.value

    # -- output (advection_solver.cc:1220-1241) -----------------------------
    def write_vtu(self, vec, time, path, stream=None):
        """VTU file with "solution" and "analytic_solution" at the support points."""
        _lib.check(self._lib.adv_write_vtu(self._h, self._ptr(vec), float(time), str(path).encode(),
                                           _stream_handle(stream)), "adv_write_vtu")

    def save_state(self, vec, time, path, stream=None):
        _lib.check(self._lib.adv_save_state(self._h, self._ptr(vec), float(time), str(path).encode(),
                                            _stream_handle(stream)), "adv_save_state")

    def load_state(self, vec, path, stream=None):
        """Fills vec from a state file of the same configuration; returns its time."""
        t = ctypes.c_double()
        _lib.check(self._lib.adv_load_state(self._h, self._ptr(vec), ctypes.byref(t), str(path).encode(),
                                            _stream_handle(stream)), "adv_load_state")
        return t.value

    # -- fused time stepping -------------------------------------------------
    def lsrk_steps(self, scheme, time, time_step, n_steps, solution, vec_ri, vec_ki, stream=None):
        _lib.check(self._lib.adv_lsrk_steps(
            self._h, int(scheme), float(time), float(time_step), int(n_steps), self._ptr(solution),
            self._ptr(vec_ri), self._ptr(vec_ki), _stream_handle(stream)), "adv_lsrk_steps")

    def lsrk_steps_host(self, scheme, time, time_step, n_steps, host_solution, solution, vec_ri, vec_ki,
                        stream=None):
        """lsrk_steps on a solution in host memory (a contiguous CPU float64
        tensor, best page-locked): copied into `solution`, advanced and copied
        back, the copies overlapped with the first and last stages.  The host
        tensor holds the result once the stream has passed the call."""
        import torch
        if not (isinstance(host_solution, torch.Tensor) and not host_solution.is_cuda
                and host_solution.dtype == torch.float64 and host_solution.is_contiguous()
                and host_solution.numel() == self.n_dofs):
            raise ValueError(f"expected a contiguous CPU float64 tensor of {self.n_dofs} entries")
        _lib.check(self._lib.adv_lsrk_steps_host(
            self._h, int(scheme), float(time), float(time_step), int(n_steps),
            ctypes.c_void_p(host_solution.data_ptr()), self._ptr(solution), self._ptr(vec_ri), self._ptr(vec_ki),
            _stream_handle(stream)), "adv_lsrk_steps_host")


class LowStorageRungeKuttaIntegrator:
    """Counterpart of the reference's LowStorageRungeKuttaIntegrator (advection_solver.cc:822-944)."""

    def __init__(self, scheme=LSRK_5_4):
        self.scheme = scheme
        self.ai, self.bi = lsrk_coefficients(scheme)

    def n_stages(self):
        return len(self.bi)

    def perform_time_step(self, pde_operator, current_time, time_step, solution, vec_ri, vec_ki,
                          stream=None):
        """One time step.  With an AdvectionOperation the whole step runs in the
        library (adv_lsrk_step); any other operator gets the reference's stage
        loop through its perform_stage."""
        if isinstance(pde_operator, AdvectionOperation) and pde_operator.slab is None:
            pde_operator.lsrk_steps(self.scheme, current_time, time_step, 1, solution, vec_ri, vec_ki,
                                    stream=stream)
            return
        bi, ai = self.bi, self.ai
        pde_operator.perform_stage(current_time, bi[0] * time_step, ai[0] * time_step, solution, vec_ri,
                                   solution, vec_ri)
        sum_previous_bi = 0.0
        for stage in range(1, len(bi)):
            c_i = sum_previous_bi + ai[stage - 1]
            pde_operator.perform_stage(current_time + c_i * time_step, bi[stage] * time_step,
                                       0.0 if stage == len(bi) - 1 else ai[stage] * time_step,
                                       vec_ri, vec_ki, solution, vec_ri)
            sum_previous_bi += bi[stage - 1]


class ImplicitSolver:
    """FGMRES(restart) with the block-Jacobi FDM preconditioner and BDF2 steps
    (the implicit path of advection_solver_implicit.cc on the GPU)."""

    def __init__(self, op, restart=30, precond_precision=PRECISION_FP32_OPERATOR):
        self.op = op
        self._lib = op._lib
        self._s = ctypes.c_void_p()
        _lib.check(self._lib.adv_solver_create(op._h, int(restart), int(precond_precision), ctypes.byref(self._s)),
                   "adv_solver_create")

    def close(self):
        if getattr(self, "_s", None):
            self._lib.adv_solver_destroy(self._s)
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def device_bytes(self):
        n = ctypes.c_int64()
        _lib.check(self._lib.adv_solver_device_bytes(self._s, ctypes.byref(n)), "adv_solver_device_bytes")
        return n.value

    def precondition(self, src, dst, mass_factor, time=0.0, stream=None):
        _lib.check(self._lib.adv_precondition(self._s, self.op._ptr(src), self.op._ptr(dst), float(mass_factor),
                                              float(time), _stream_handle(stream)), "adv_precondition")

    def fgmres(self, mass_factor, time, rhs, x, rel_tol=1e-10, max_iterations=1000, stream=None):
        """Solve (mass_factor M - L) x = rhs from the initial guess in x; returns (iterations, relative residual)."""
        its, res = ctypes.c_int(), ctypes.c_double()
        _lib.check(self._lib.adv_fgmres(self._s, float(mass_factor), float(time), self.op._ptr(rhs), self.op._ptr(x),
                                        float(rel_tol), int(max_iterations), ctypes.byref(its), ctypes.byref(res),
                                        _stream_handle(stream)), "adv_fgmres")
        return its.value, res.value

    def bdf2_step(self, t_new, dt, first_step, u_n, u_nm1, u_new, rel_tol=1e-10, stream=None):
        """One BDF2 step (implicit Euler when first_step); returns the FGMRES iterations."""
        its = ctypes.c_int()
        _lib.check(self._lib.adv_bdf2_step(self._s, float(t_new), float(dt), int(bool(first_step)),
                                           self.op._ptr(u_n), self.op._ptr(u_nm1) if u_nm1 is not None else None,
                                           self.op._ptr(u_new), float(rel_tol), ctypes.byref(its),
                                           _stream_handle(stream)), "adv_bdf2_step")
        return its.value
