"""ctypes binding of libqgybj.so (include/qgybj.h).

The library is loaded from this directory.  There is no fallback: when the
shared object is missing or fails to load, importing this module raises.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libqgybj.so"

QG_OK, QG_ERR_ARG, QG_ERR_CUDA, QG_ERR_NONFINITE, QG_ERR_PIVOT, QG_ERR_TIMEOUT, QG_ERR_UNSUPPORTED, QG_ERR_NOMEM = range(8)
QG_PREC_FP64, QG_PREC_MIXED = 0, 1
FIELDS = {"q": 0, "qo": 1, "BR": 2, "BI": 3, "BRo": 4, "BIo": 5, "psi": 6, "AR": 7, "AI": 8, "CR": 9, "CI": 10,
          "qstar": 11}
STATUS_NAMES = {0: "QG_OK", 1: "QG_ERR_ARG", 2: "QG_ERR_CUDA", 3: "QG_ERR_NONFINITE", 4: "QG_ERR_PIVOT",
                5: "QG_ERR_TIMEOUT", 6: "QG_ERR_UNSUPPORTED", 7: "QG_ERR_NOMEM"}

EXPORTS = (
    "qg_config_defaults", "qg_create", "qg_destroy", "qg_last_error", "qg_set_state", "qg_get_state",
    "qg_init_state", "qg_step", "qg_steps_async", "qg_synchronize", "qg_get_stream", "qg_diagnostics_fp64",
    "qg_fft_r2c", "qg_fft_c2r", "qg_convol_waqg", "qg_refraction_waqg", "qg_compute_qw", "qg_psi_solver",
    "qg_A_solver_ybj_plus", "qg_profile_step", "qg_fft_c2r_noalloc",
    "qg_ensemble_create", "qg_ensemble_member", "qg_ensemble_step", "qg_ensemble_synchronize",
    "qg_ensemble_get_stream", "qg_ensemble_destroy", "qg_ensemble_last_error", "qg_autotune",
    "qg_adjoint_run", "qg_adjoint_step", "qg_dump_psi", "qg_dump_la",
    "qg_omega_eqn_rhs", "qg_omega_equation", "qg_omega", "qg_ensemble_set_lanes",
    "qg_selftest_conversions", "qg_selftest_wait", "qg_ensemble_profile_step",
    "qg_diagnostics_fp64_async", "qg_diagnostics_fp64_wait",
)
KERNEL_CLASSES = ("dissipation", "col_inv", "row_main", "col_update", "row_qw", "col_qw", "solve", "solve_A")


class QgConfig(C.Structure):
    _fields_ = [
        ("n1", C.c_int), ("n2", C.c_int), ("n3", C.c_int), ("precision", C.c_int), ("device", C.c_int),
        ("ybj_plus", C.c_int), ("fixed_flow", C.c_int), ("no_feedback", C.c_int), ("passive_scalar", C.c_int),
        ("linear", C.c_int), ("no_dispersion", C.c_int), ("inviscid", C.c_int),
        ("dz", C.c_double), ("Bu", C.c_double), ("Ro", C.c_double), ("W2F", C.c_double),
        ("delt", C.c_double), ("gamma", C.c_double),
        ("nuh1", C.c_double), ("nuh2", C.c_double), ("nuh1w", C.c_double), ("nuh2w", C.c_double),
        ("ilap1", C.c_int), ("ilap2", C.c_int), ("ilap1w", C.c_int), ("ilap2w", C.c_int),
        ("nuz", C.c_double),
        ("a_ell_ut", C.POINTER(C.c_double)), ("rho_ut", C.POINTER(C.c_double)),
        ("rho_st", C.POINTER(C.c_double)), ("r_2ut", C.POINTER(C.c_double)),
        ("levels_per_batch", C.c_int), ("use_graphs", C.c_int), ("solve_columns", C.c_int),
    ]


class QgTuning(C.Structure):
    _fields_ = [("levels_per_batch", C.c_int), ("ms_per_step", C.c_double), ("ncandidates", C.c_int),
                ("candidates", C.c_int * 16), ("candidate_ms", C.c_double * 16),
                ("solve_columns", C.c_int), ("nsolve", C.c_int), ("solve_candidates", C.c_int * 4),
                ("solve_candidate_ms", C.c_double * 4)]


class QgEnergy(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("wke", "wpe", "wce", "ke", "pe", "zeta2", "omegah2")]


_lib = None


def lib() -> C.CDLL:
    """Load libqgybj.so (raises OSError when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise OSError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
    L = C.CDLL(str(LIB_PATH))
    vp, dp, ip = C.c_void_p, C.POINTER(C.c_double), C.c_int
    sig = {
        "qg_config_defaults": (ip, [C.POINTER(QgConfig)]),
        "qg_create": (ip, [C.POINTER(QgConfig), C.POINTER(vp)]),
        "qg_destroy": (ip, [vp]),
        "qg_last_error": (C.c_char_p, [vp]),
        "qg_set_state": (ip, [vp, ip, vp, ip, ip]),
        "qg_get_state": (ip, [vp, ip, vp, ip, ip]),
        "qg_init_state": (ip, [vp, ip, ip]),
        "qg_step": (ip, [vp, ip]),
        "qg_steps_async": (ip, [vp, ip, ip]),
        "qg_synchronize": (ip, [vp]),
        "qg_get_stream": (ip, [vp, C.POINTER(vp)]),
        "qg_diagnostics_fp64": (ip, [vp, C.POINTER(QgEnergy)]),
        "qg_fft_r2c": (ip, [vp, vp, vp, ip]),
        "qg_fft_c2r": (ip, [vp, vp, vp, ip]),
        "qg_convol_waqg": (ip, [vp] + [vp] * 8 + [ip]),
        "qg_refraction_waqg": (ip, [vp] + [vp] * 5 + [ip]),
        "qg_compute_qw": (ip, [vp, vp, vp, vp, ip]),
        "qg_psi_solver": (ip, [vp, vp, vp]),
        "qg_A_solver_ybj_plus": (ip, [vp, vp, vp, vp]),
        "qg_profile_step": (ip, [vp, ip, dp, C.POINTER(C.c_int), ip]),
        "qg_fft_c2r_noalloc": (ip, [vp, vp, ip, ip, vp]),
        "qg_selftest_conversions": (ip, [ip, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
        "qg_selftest_wait": (ip, [vp]),
        "qg_ensemble_create": (ip, [C.POINTER(QgConfig), ip, C.POINTER(vp)]),
        "qg_ensemble_member": (ip, [vp, ip, C.POINTER(vp)]),
        "qg_ensemble_step": (ip, [vp, ip, ip]),
        "qg_ensemble_synchronize": (ip, [vp]),
        "qg_ensemble_get_stream": (ip, [vp, C.POINTER(vp)]),
        "qg_ensemble_destroy": (ip, [vp]),
        "qg_ensemble_last_error": (C.c_char_p, [vp]),
        "qg_ensemble_profile_step": (ip, [vp, ip, C.POINTER(C.c_double), C.POINTER(C.c_int), ip]),
        "qg_diagnostics_fp64_async": (ip, [vp]),
        "qg_diagnostics_fp64_wait": (ip, [vp, C.POINTER(QgEnergy)]),
        "qg_autotune": (ip, [C.POINTER(QgConfig), ip, C.POINTER(QgTuning)]),
        "qg_adjoint_run": (ip, [vp, vp, vp, vp, ip, ip, ip, dp, vp, vp, vp]),
        "qg_adjoint_step": (ip, [vp, ip, vp, vp, vp, vp]),
        "qg_dump_psi": (ip, [vp, vp, ip, ip, C.c_double, C.c_double]),
        "qg_dump_la": (ip, [vp, vp, vp, ip, ip, C.c_double, ip]),
        "qg_omega_eqn_rhs": (ip, [vp, vp, vp]),
        "qg_omega_equation": (ip, [vp, vp, vp]),
        "qg_omega": (ip, [vp, vp]),
        "qg_ensemble_set_lanes": (ip, [vp, ip]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


class QgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def check(status: int, handle=None) -> None:
    if status != QG_OK:
        msg = lib().qg_last_error(handle)
        raise QgError(status, msg.decode() if msg else "")


def ptr(a) -> int | None:
    """Address of a numpy array (host) or a torch tensor (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags.c_contiguous:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    raise TypeError(type(a))
