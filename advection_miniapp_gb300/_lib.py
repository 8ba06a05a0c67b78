"""ctypes binding of libadvection_gb300.so (the C ABI in include/advection_gb300.h).

Loading never falls back to anything: if the library is missing or does not
load, the error says so and no computation is possible.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libadvection_gb300.so")

ADV_OK = 0
ERRORS = {1: "invalid argument", 2: "out of memory", 3: "CUDA error", 4: "aliasing",
          5: "not converged", 6: "timeout"}

MESH_CARTESIAN, MESH_DEFORMED = 0, 1
VELOCITY_CONSTANT, VELOCITY_ROTATING = 0, 1
IC_SINE_GAUSS, IC_BLOB, IC_WAVE = 0, 1, 2
BOUNDARY_ZERO, BOUNDARY_EXACT = 0, 1
PRECISION_FP64, PRECISION_FP32_OPERATOR, PRECISION_FP32_INCREMENT = 0, 1, 2
LSRK_3_3, LSRK_5_4, LSRK_7_4, LSRK_9_5 = 0, 1, 2, 3
FORM_AUTO, FORM_NODAL, FORM_COLLOCATION, FORM_COLLOCATION_NO_TRACES = 0, 1, 2, 3


class AdvConfig(ctypes.Structure):
    """Mirror of adv_config."""
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
        ("precision", ctypes.c_int32),
        ("fused_form", ctypes.c_int32),
        ("anchor_interval", ctypes.c_int32),
        ("reserved1", ctypes.c_int32 * 5),
    ]


# name -> (restype, argtypes)
_P, _D, _I, _I64 = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int64
_DP = ctypes.POINTER(ctypes.c_double)
SIGNATURES = {
    "adv_config_default": (None, [ctypes.POINTER(AdvConfig)]),
    "adv_create": (_I, [ctypes.POINTER(AdvConfig), ctypes.POINTER(_P)]),
    "adv_destroy": (_I, [_P]),
    "adv_last_error": (ctypes.c_char_p, []),
    "adv_n_dofs": (_I, [_P, ctypes.POINTER(_I64)]),
    "adv_n_cells": (_I, [_P, ctypes.POINTER(_I64)]),
    "adv_device_bytes": (_I, [_P, ctypes.POINTER(_I64)]),
    "adv_alloc_vector": (_I, [_P, ctypes.POINTER(_P)]),
    "adv_free_vector": (_I, [_P, _P]),
    "adv_apply": (_I, [_P, _P, _P, _D, _P]),
    "adv_perform_stage": (_I, [_P, _D, _D, _D, _P, _P, _P, _P, _P]),
    "adv_lsrk_step": (_I, [_P, _I, _D, _D, _P, _P, _P, _P]),
    "adv_lsrk_steps": (_I, [_P, _I, _D, _D, _I, _P, _P, _P, _P]),
    "adv_lsrk_steps_host": (_I, [_P, _I, _D, _D, _I, _P, _P, _P, _P, _P]),
    "adv_lsrk_coefficients": (_I, [_I, _DP, _DP, ctypes.POINTER(_I)]),
    "adv_project": (_I, [_P, _D, _P, _P]),
    "adv_mass_energy": (_I, [_P, _P, _DP, _P]),
    "adv_l2_error": (_I, [_P, _P, _D, _DP, _P]),
    "adv_time_step": (_I, [_P, _D, _DP]),
    "adv_copy_to_host": (_I, [_P, _P, _P, _P]),
    "adv_copy_from_host": (_I, [_P, _P, _P, _P]),
    "adv_launch_count": (_I, [_P, ctypes.POINTER(_I64)]),
    "adv_measure_fma_peak": (_I, [_I, _DP, _P]),
    "adv_perform_stage_noalloc": (_I, [_P, _D, _D, _D, _P, _P, _P, _P, _P]),
    "adv_fdm_tables": (_I, [_I, _D, _I, _DP, _DP, _DP, _DP, _DP]),
    "adv_vmult": (_I, [_P, _P, _P, _D, _D, _P]),
    "adv_apply_mass": (_I, [_P, _P, _P, _P]),
    "adv_solver_create": (_I, [_P, _I, _I, ctypes.POINTER(_P)]),
    "adv_solver_destroy": (_I, [_P]),
    "adv_solver_device_bytes": (_I, [_P, ctypes.POINTER(_I64)]),
    "adv_precondition": (_I, [_P, _P, _P, _D, _D, _P]),
    "adv_fgmres": (_I, [_P, _D, _D, _P, _P, _D, _I, ctypes.POINTER(_I), _DP, _P]),
    "adv_bdf2_step": (_I, [_P, _D, _D, _I, _P, _P, _P, _D, ctypes.POINTER(_I), _P]),
    "adv_create_slab": (_I, [ctypes.POINTER(AdvConfig), _I, _I, ctypes.POINTER(_P)]),
    "adv_slab_layout": (_I, [ctypes.POINTER(AdvConfig), _I, _I, ctypes.POINTER(_I64)]),
    "adv_set_timing": (_I, [_P, _I]),
    "adv_timing": (_I, [_P, _DP, ctypes.POINTER(_I64)]),
    "adv_write_vtu": (_I, [_P, _P, _D, ctypes.c_char_p, _P]),
    "adv_write_vtu_host": (_I, [ctypes.POINTER(AdvConfig), _DP, _D, ctypes.c_char_p]),
    "adv_save_state": (_I, [_P, _P, _D, ctypes.c_char_p, _P]),
    "adv_load_state": (_I, [_P, _P, _DP, ctypes.c_char_p, _P]),
    "adv_server_create": (_I, [_I64, _I, _I, _I, ctypes.POINTER(_P)]),
    "adv_server_destroy": (_I, [_P]),
    "adv_server_set_policy": (_I, [_P, _I]),
    "adv_server_submit": (_I, [_P, ctypes.POINTER(AdvConfig), _D, _D, ctypes.POINTER(_I64)]),
    "adv_server_poll": (_I, [_P, ctypes.POINTER(_I)]),
    "adv_server_drain": (_I, [_P]),
    "adv_server_cancel": (_I, [_P, _I64]),
    "adv_server_result": (_I, [_P, _I64, ctypes.POINTER(_I), _DP, _DP, ctypes.POINTER(_I), _DP]),
    "adv_server_solution": (_I, [_P, _I64, _DP, _I64]),
    "adv_server_stats": (_I, [_P, ctypes.POINTER(_I64)]),
}

_lib = None


def load():
    """Load libadvection_gb300.so; raises if it is missing (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with advection_miniapp_gb300.build.build() "
            "(the CUDA extension is required; there is no CPU fallback)")
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class AdvError(RuntimeError):
    def __init__(self, code, where):
        msg = load().adv_last_error().decode(errors="replace")
        super().__init__(f"{where} failed ({ERRORS.get(code, code)}): {msg}")
        self.code = code


def check(code, where):
    if code != ADV_OK:
        raise AdvError(code, where)
