"""ctypes front end of oracle/ref_runner.c (TEST INFRASTRUCTURE ONLY): runs the
reference's own kernels (cubins built from the reference sources by
oracle/ref_build.py) on the GPU, to produce golden outputs that pin the oracle."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REF_DIR = HERE / "_ref"


class RRParams(C.Structure):
    _fields_ = [("max_iter", C.c_int), ("reset_iter", C.c_int), ("max_update_norm", C.c_float),
                ("rho_0", C.c_float), ("tau", C.c_float), ("w_reg", C.c_float), ("alpha", C.c_float),
                ("p", C.c_float), ("C", C.c_float)]


def available() -> bool:
    return all((REF_DIR / f"{u}.cubin").exists() for u in ("solver", "vector_fields", "reductor", "scalar_fields",
                                                            "volume"))


def _lib():
    path = REF_DIR / "libref_runner.so"
    if not path.exists():
        from oracle import ref_build
        ref_build.build_runner()
    lib = C.CDLL(str(path))
    lib.rr_register.restype = C.c_int
    lib.rr_field_op.restype = C.c_int
    lib.rr_last_error.restype = C.c_char_p
    return lib


def _field_op(op, a, b, sweeps=0):
    lib = _lib()
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    _, z, y, x = a.shape
    out = np.empty_like(a)
    dims = (C.c_int * 3)(x, y, z)
    p = lambda v: v.ctypes.data_as(C.c_void_p)  # noqa: E731
    if lib.rr_field_op(str(REF_DIR).encode(), dims, op, int(sweeps), p(a), p(b), p(out)) != 0:
        raise RuntimeError("reference run failed: " + lib.rr_last_error().decode())
    return out


def estimate_inverse(psi, psi_inv, sweeps=48):
    """The reference's DeformationField::get_inverse (vector_fields.cpp:96-103): `sweeps`
    launches of estimate_inverse_kernel, psi_inv (3 planes) updated in place; returns it."""
    return _field_op(0, psi, psi_inv, sweeps)


def interpolate_gradient(field, psi):
    """The reference's interpolate_gradient: field (3 planes) sampled at psi."""
    return _field_op(1, psi, field)


def register(params, T, labT, S, labS, timing=False):
    """One registration with the reference kernels; params has the Params fields.
    With timing=True the result also holds ms_operator (device time of the whole
    FastReg::operator() sequence, input upload to the last warp) and ms_estimate_psi."""
    lib = _lib()
    T = np.ascontiguousarray(T, np.float32)
    S = np.ascontiguousarray(S, np.float32)
    labT = np.ascontiguousarray(labT, np.int16)
    labS = np.ascontiguousarray(labS, np.int16)
    z, y, x = T.shape
    P = RRParams(int(params.max_iter), int(params.reset_iter), params.max_update_norm, params.rho_0, params.tau,
                 params.w_reg, params.alpha, params.p, params.C)
    dims = (C.c_int * 3)(x, y, z)
    oT, oS = np.empty_like(T), np.empty_like(S)
    olT, olS = np.empty_like(labT), np.empty_like(labS)
    psi = np.empty((3, z, y, x), np.float32)
    pinv = np.empty((3, z, y, x), np.float32)
    n = max(int(params.max_iter), 1)
    tn = np.zeros(n, np.float32)
    ti = np.zeros(n, np.int64)
    ms = np.zeros(2, np.float32)
    p = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    ran = lib.rr_register(str(REF_DIR).encode(), dims, C.byref(P), p(T), p(labT), p(S), p(labS), p(oT), p(olT),
                          p(oS), p(olS), p(psi), p(pinv), p(tn), p(ti), p(ms))
    if ran < 0:
        raise RuntimeError("reference run failed: " + lib.rr_last_error().decode())
    out = dict(out_T=oT, out_labT=olT, out_S=oS, out_labS=olS, psi=psi, psi_inv=pinv, iterations=int(ran),
               trace_norm=tn[:ran], trace_idx=ti[:ran])
    if timing:
        out["ms_operator"] = float(ms[0])
        out["ms_estimate_psi"] = float(ms[1])
    return out
