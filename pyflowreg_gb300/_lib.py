"""ctypes binding of the C ABI in ``include/flowreg_gb300.h``.

The shared library is built in-tree (``pyflowreg_gb300/_build``) by
``pyflowreg_gb300.build``.  There is no fallback: if the library is missing or
fails to load, every entry point raises.
"""

from __future__ import annotations

import ctypes
import os
import threading

from . import build as _build

FRG_OK = 0
FRG_EINVAL = 1
FRG_ENOMEM = 2
FRG_ECUDA = 3
FRG_EUNSUPPORTED = 4
FRG_ECALLBACK = 5
FRG_MAX_CHANNELS = 8
FRG_MAX_GNC_STAGES = 16

_lock = threading.Lock()
_lib = None


class FrgParams(ctypes.Structure):
    _fields_ = [
        ("alpha_x", ctypes.c_double),
        ("alpha_y", ctypes.c_double),
        ("eta", ctypes.c_double),
        ("levels", ctypes.c_int),
        ("min_level", ctypes.c_int),
        ("iterations", ctypes.c_int),
        ("update_lag", ctypes.c_int),
        ("a_smooth", ctypes.c_double),
        ("a_data", ctypes.c_double * FRG_MAX_CHANNELS),
        ("const_assumption", ctypes.c_int),
        ("omega", ctypes.c_double),
        ("precision", ctypes.c_int),
        ("gnc_stages", ctypes.c_int),
        ("gnc_schedule", ctypes.c_double * FRG_MAX_GNC_STAGES),
        ("warping_steps", ctypes.c_int),
    ]


FRG_FP32 = 0
FRG_FP64_REFERENCE = 1


# frg_level_solver_fn: (user, level, frame, m, n, K, J, W, u, v, alpha_x, alpha_y, hx, hy, du, dv) -> int
LEVEL_SOLVER_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                   ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p)


class FrgError(RuntimeError):
    """A C-ABI call returned a status other than FRG_OK."""


def _sig(lib, name, restype, argtypes):
    fn = getattr(lib, name)
    fn.restype = restype
    fn.argtypes = argtypes
    return fn


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Loads (building first if needed) and returns the ctypes library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise ImportError(f"GB300 backend library not built: {path}")
        lib = ctypes.CDLL(path)
        P, I, D, S = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_size_t
        pI, pD, pF = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_float)
        pP = ctypes.POINTER(FrgParams)
        _sig(lib, "frg_version", I, [])
        _sig(lib, "frg_last_error", ctypes.c_char_p, [])
        _sig(lib, "frg_schedule", I, [pP, I, I, I, pI, pI, pD, pD])
        _sig(lib, "frg_resize_tables", I, [I, I, D, I, pI, pF])
        _sig(lib, "frg_iteration_passes", I, [I, I, I, pI, pI])
        _sig(lib, "frg_plan_create", I, [pP, I, I, I, I, ctypes.POINTER(P)])
        _sig(lib, "frg_plan_destroy", None, [P])
        _sig(lib, "frg_plan_device_bytes", S, [P])
        _sig(lib, "frg_plan_num_levels", I, [P])
        _sig(lib, "frg_plan_level_info", I, [P, I, pI, pI, pD, pD])
        _sig(lib, "frg_plan_set_level_tables", I, [P, I, I, I, pI, pF, pI, pF])
        _sig(lib, "frg_plan_set_level_tuning", I, [P, I, I, I])
        _sig(lib, "frg_plan_level_tuning", I, [P, I, pI, pI, pI, pI])
        _sig(lib, "frg_plan_set_level_variant", I, [P, I, I])
        _sig(lib, "frg_plan_set_level_solver", I, [P, LEVEL_SOLVER_FN, P])
        _sig(lib, "frg_plan_level_variant", I, [P, I, pI, pI])
        _sig(lib, "frg_launch_count", ctypes.c_longlong, [])
        _sig(lib, "frg_plan_set_profiling", I, [P, I])
        _sig(lib, "frg_plan_profile", I, [P, ctypes.POINTER(ctypes.c_longlong), pD, pD])
        _sig(lib, "frg_set_reference", I, [P, P, P, P])
        _sig(lib, "frg_get_displacement", I, [P, I, P, P, P, P])
        _sig(lib, "frg_get_displacement_f64", I, [P, I, P, P, P, P])
        _sig(lib, "frg_imregister", I, [I, I, I, I, P, P, P, I, P, P])
        _sig(lib, "frg_level_solve", I, [I, I, I, P, P, P, P, D, D, I, I, pD, D, D, D, D, P, P, P])
        _sig(lib, "frg_level_solve_noalloc", I, [I, I, I, P, P, P, P, D, D, I, I, pD, D, D, D, D, P, P, P])
        _sig(lib, "frg_level_solve_noalloc_capacity", S, [])
        _sig(lib, "frg_level_solve_f64", I, [I, I, I, P, P, P, P, D, D, I, I, pD, D, D, D, D, D, P, P, P])
        _sig(lib, "frg_resize", I, [I, I, I, P, I, I, P, P])
        _sig(lib, "frg_motion_tensor", I, [I, I, P, P, D, D, I, P, P])
        _sig(lib, "frg_median5", I, [I, I, P, P, P])
        _sig(lib, "frg_median5_f64", I, [I, I, P, P, P])
        _sig(lib, "frg_pow_f64", I, [ctypes.c_longlong, P, D, P, P])
        _sig(lib, "frg_host_register", I, [P, ctypes.c_longlong])
        _sig(lib, "frg_host_unregister", I, [P])
        _sig(lib, "frg_preprocess", I, [I, I, I, I, P, pD, pD, P, pI, P, pI, P, pI, I, I, P, P, P])
        _sig(lib, "frg_preprocess_f64", I, [I, I, I, I, P, pD, pD, P, pI, P, pI, P, pI, I, P, P, P])
        _sig(lib, "frg_flow_post_workspace", S, [I, I, I])
        _sig(lib, "frg_flow_post", I, [I, I, I, P, P, P, P, P])
        _sig(lib, "frg_diff_plan_create", I, [pP, I, I, I, I, I, ctypes.POINTER(P)])
        _sig(lib, "frg_diff_plan_destroy", None, [P])
        _sig(lib, "frg_diff_plan_device_bytes", S, [P])
        _sig(lib, "frg_diff_plan_num_levels", I, [P])
        _sig(lib, "frg_diff_set_level_tables", I, [P, I, I, I, pI, pF, pI, pF])
        _sig(lib, "frg_diff_set_weight", I, [P, P, P])
        _sig(lib, "frg_diff_forward", I, [P, I, D, D, P, P, P, P, P])
        _sig(lib, "frg_diff_backward", I, [P, P, P, P, P, I, P])
        _sig(lib, "frg_diff_warp", I, [I, I, I, I, I, P, P, P, P, P])
        _sig(lib, "frg_diff_warp_backward", I, [I, I, I, I, I, P, P, P, P, P, P, P])
        _lib = lib
        return lib


def check(rc: int, what: str = "") -> None:
    """Maps a status code to the exception the reference would raise."""
    if rc == FRG_OK:
        return
    msg = (load().frg_last_error() or b"").decode(errors="replace")
    text = f"{what}: {msg}" if what else msg
    if rc == FRG_EINVAL:
        raise ValueError(text)
    if rc == FRG_EUNSUPPORTED:
        raise NotImplementedError(text)
    if rc == FRG_ENOMEM:
        raise MemoryError(text)
    raise FrgError(f"[status {rc}] {text}")
