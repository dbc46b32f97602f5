"""ctypes binding of the C ABI declared in include/fastreg_gb300.h.

The shared library is built in-tree by fastreg_gb300.build; loading fails loudly
when it is missing -- there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_lib" / "libfastreg_gb300.so"

FR_OK = 0
FR_ERR_INVALID_ARG = 1
FR_ERR_CUDA = 2
FR_ERR_ALLOC = 3
FR_ERR_IO = 4
FR_ERR_PARSE = 5
FR_ERR_STATE = 6
FR_ERR_NUMERIC = 7

FR_SOLVER_REFERENCE = 0
FR_SOLVER_SOBOLEV = 1

FR_FIELD_PSI = 0
FR_FIELD_PSI_INV = 1
FR_FIELD_V = 2
FR_FIELD_RHO = 3

FR_MAX_LABELS = 256


class fr_params(C.Structure):
    _fields_ = [
        ("volume_dims", C.c_int * 3),
        ("volume_size", C.c_float * 3),
        ("no_labels", C.c_int),
        ("max_iter", C.c_int),
        ("max_update_norm", C.c_float),
        ("rho_0", C.c_float),
        ("tau", C.c_float),
        ("w_reg", C.c_float),
        ("alpha", C.c_float),
        ("p", C.c_float),
        ("C", C.c_float),
        ("reset_iter", C.c_int),
        ("verbosity", C.c_int),
        ("solver", C.c_int),
        ("smooth_sigma", C.c_float),
        ("smooth_width", C.c_int),
        ("damping", C.c_float),
        ("step", C.c_float),
        ("keep_state", C.c_int),
        ("autotune", C.c_int),
        ("staging", C.c_int),
    ]


class fr_pair(C.Structure):
    _fields_ = [
        ("dims", C.c_int * 3),
        ("img_T", C.c_void_p),
        ("lab_T", C.c_void_p),
        ("img_S", C.c_void_p),
        ("lab_S", C.c_void_p),
    ]


class fr_stats(C.Structure):
    _fields_ = [
        ("iterations", C.c_int),
        ("converged", C.c_int),
        ("last_max_update_norm", C.c_float),
        ("last_max_update_voxel", C.c_int64),
        ("e_data", C.c_double),
        ("e_reg", C.c_double),
        ("energy", C.c_double),
        ("folds", C.c_int64),
        ("no_labels", C.c_int),
        ("dice", C.c_double * FR_MAX_LABELS),
        ("dice_all", C.c_double),
        ("dice_out_of_range", C.c_int64),
        ("dice_inter", C.c_int64 * FR_MAX_LABELS),
        ("dice_count", C.c_int64 * FR_MAX_LABELS),
    ]


# (name, restype, argtypes) of every exported entry point; the CPU tests check
# that the library exports exactly these names.
SIGNATURES = [
    ("fr_params_default", C.c_int, [C.POINTER(fr_params)]),
    ("fr_params_parse_ini", C.c_int, [C.c_char_p, C.POINTER(fr_params)]),
    ("fr_params_load_ini", C.c_int, [C.c_char_p, C.POINTER(fr_params)]),
    ("fr_create", C.c_int, [C.POINTER(fr_params), C.POINTER(C.c_void_p)]),
    ("fr_destroy", C.c_int, [C.c_void_p]),
    ("fr_register", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fr_register_batch", C.c_int, [C.c_void_p, C.POINTER(fr_pair), C.c_int, C.c_void_p]),
    ("fr_get_stats", C.c_int, [C.c_void_p, C.c_int, C.POINTER(fr_stats)]),
    ("fr_get_trace", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    ("fr_get_field", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("fr_set_field", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("fr_begin", C.c_int, [C.c_void_p, C.POINTER(fr_pair), C.c_int, C.c_void_p]),
    ("fr_step", C.c_int, [C.c_void_p, C.c_int, C.c_float, C.c_void_p]),
    ("fr_finish", C.c_int, [C.c_void_p, C.c_void_p]),
    ("fr_time_kernels", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_int), C.c_void_p]),
    ("fr_warp", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.c_void_p, C.c_void_p, C.c_void_p]),
    ("fr_set_pair_w_reg", C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    ("fr_tile_shape", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("fr_tile_staging", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    ("fr_estimate_inverse", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.c_int, C.c_void_p]),
    ("fr_interpolate_field", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.c_void_p, C.c_void_p]),
    ("fr_sobolev_loss_grad", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.c_void_p, C.c_float, C.c_int,
                                       C.c_int, C.c_float, C.c_float, C.c_float, C.c_int, C.POINTER(C.c_double),
                                       C.c_void_p, C.POINTER(C.c_double), C.c_void_p]),
    ("fr_warp_adjoint", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int), C.c_void_p, C.c_void_p,
                                  C.c_void_p]),
    ("fr_stats_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int),
                                   C.c_int, C.c_float, C.POINTER(fr_stats), C.c_void_p]),
    ("fr_selftest_wait_limit", C.c_int, [C.POINTER(C.c_double), C.c_void_p]),
    ("fr_last_error", C.c_char_p, [C.c_void_p]),
    ("fr_status_string", C.c_char_p, [C.c_int]),
    ("fr_abi_version", C.c_int, []),
]

_lib = None


def load() -> C.CDLL:
    """Load the native library (built by fastreg_gb300.build); raises if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(
            f"fastreg_gb300 native library not found at {LIB_PATH}; "
            "build it with `python -m fastreg_gb300.build` (there is no CPU fallback)")
    lib = C.CDLL(str(LIB_PATH))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class FastRegError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} [status {status}]")
        self.status = status


def check(status: int, handle=None, what: str = "") -> None:
    if status == FR_OK:
        return
    lib = load()
    msg = lib.fr_last_error(handle)
    msg = msg.decode() if msg else ""
    kind = lib.fr_status_string(status).decode()
    raise FastRegError(status, f"{what}: {kind}: {msg}" if what else f"{kind}: {msg}")
