"""numpy front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by the tests, by __graft_entry__.smoke() and by the CPU-baseline leg of
bench.py -- never by the product library.  Arrays are (Z, Y, X) float32 volumes
and (3, Z, Y, X) vector fields; ``prec=64`` selects the FP64 build.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_libs: dict = {}


class RefCoef32(C.Structure):
    _fields_ = [("alpha", C.c_float), ("f1", C.c_float), ("m2", C.c_float), ("tau", C.c_float),
                ("w_reg", C.c_float)]


class RefCoef64(C.Structure):
    _fields_ = [("alpha", C.c_double), ("f1", C.c_double), ("m2", C.c_double), ("tau", C.c_double),
                ("w_reg", C.c_double)]


def _ref_params_type(real):
    class RefParams(C.Structure):
        _fields_ = [("max_iter", C.c_int), ("reset_iter", C.c_int), ("max_update_norm", real), ("rho_0", real),
                    ("tau", real), ("w_reg", real), ("alpha", real), ("p", real), ("C", real),
                    ("keep_state", C.c_int)]
    return RefParams


def _sob_params_type(real):
    class SobParams(C.Structure):
        _fields_ = [("max_iter", C.c_int), ("max_update_norm", real), ("damping", real), ("step", real),
                    ("sigma", real), ("width", C.c_int), ("lam", real)]
    return SobParams


def _sobgrad_params_type(real):
    class SobGradParams(C.Structure):
        _fields_ = [("iters", C.c_int), ("damping", real), ("step", real), ("sigma", real), ("width", C.c_int)]
    return SobGradParams


RefParams32, RefParams64 = _ref_params_type(C.c_float), _ref_params_type(C.c_double)
SobParams32, SobParams64 = _sob_params_type(C.c_float), _sob_params_type(C.c_double)
SobGradParams32, SobGradParams64 = _sobgrad_params_type(C.c_float), _sobgrad_params_type(C.c_double)


class Stats(C.Structure):
    _fields_ = [("e_data", C.c_double), ("e_reg", C.c_double), ("folds", C.c_int64),
                ("dice_inter", C.c_int64 * 256), ("dice_count", C.c_int64 * 256), ("dice_out_of_range", C.c_int64)]


def lib(prec: int = 32):
    if prec not in _libs:
        path = HERE / "_build" / f"libfr_oracle{prec}.so"
        if not path.exists():
            raise RuntimeError(f"oracle library {path} missing; run `python oracle/build.py`")
        _libs[prec] = C.CDLL(str(path))
    return _libs[prec]


def _dt(prec):
    return np.float32 if prec == 32 else np.float64


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _dims(shape):
    z, y, x = shape[-3:]
    return (C.c_int * 3)(x, y, z)


def _f(a, prec):
    return np.ascontiguousarray(a, dtype=_dt(prec))


def ref_coef(alpha, t, p, Cc, tau, w_reg, prec=32):
    L = lib(prec)
    real = C.c_float if prec == 32 else C.c_double
    k = RefCoef32() if prec == 32 else RefCoef64()
    fn = getattr(L, f"fro{prec}_ref_coef")
    fn.argtypes = [real] * 6 + [C.c_void_p]
    fn(alpha, t, p, Cc, tau, w_reg, C.byref(k))
    return k


def ref_laplacian(psi, prec=32):
    psi = _f(psi, prec)
    out = np.empty_like(psi)
    getattr(lib(prec), f"fro{prec}_ref_laplacian")(_dims(psi.shape), _p(psi), _p(out))
    return out


def ref_pass_a(k, S, T, first_iter, rho, v, pinv, L, prec=32):
    S, T, rho, v, pinv, L = (_f(a, prec) for a in (S, T, rho, v, pinv, L))
    rho_n, v_n, pinv_n = rho.copy(), v.copy(), pinv.copy()
    getattr(lib(prec), f"fro{prec}_ref_pass_a")(_dims(S.shape), C.byref(k), _p(S), _p(T), C.c_int(int(first_iter)),
                                               _p(rho), _p(v), _p(pinv), _p(L), _p(rho_n), _p(v_n), _p(pinv_n))
    return rho_n, v_n, pinv_n


def ref_pass_b(alpha, v, psi, prec=32):
    v = _f(v, prec)
    psi = _f(psi, prec).copy()
    real = C.c_float if prec == 32 else C.c_double
    mx = real()
    am = C.c_int64()
    fn = getattr(lib(prec), f"fro{prec}_ref_pass_b")
    fn.argtypes = [C.c_void_p, real, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    fn(_dims(v.shape), alpha, _p(v), _p(psi), C.byref(mx), C.byref(am))
    return psi, float(mx.value), int(am.value)


def warp(pos, img, lab=None, prec=32):
    pos, img = _f(pos, prec), _f(img, prec)
    out = np.empty_like(img)
    out_lab = None
    if lab is not None:
        lab = np.ascontiguousarray(lab, dtype=np.int16)
        out_lab = np.empty_like(lab)
    getattr(lib(prec), f"fro{prec}_warp")(_dims(img.shape), _p(pos), _p(img), _p(lab) if lab is not None else None,
                                          _p(out), _p(out_lab) if lab is not None else None)
    return (out, out_lab) if lab is not None else out


def estimate_inverse(psi, psi_inv, sweeps=48, prec=32):
    """The reference's estimate_inverse: `sweeps` in-place passes of
    psi_inv <- -psi o psi_inv (3-plane fields); returns the final psi_inv."""
    psi = _f(psi, prec)
    out = _f(psi_inv, prec).copy()
    getattr(lib(prec), f"fro{prec}_estimate_inverse")(_dims(psi.shape[1:]), _p(psi), _p(out), int(sweeps))
    return out


def interpolate_field(field, pos, prec=32):
    """The reference's interpolate_gradient: a 3-plane field sampled at pos."""
    field, pos = _f(field, prec), _f(pos, prec)
    out = np.empty_like(field)
    getattr(lib(prec), f"fro{prec}_interpolate_field")(_dims(field.shape[1:]), _p(field), _p(pos), _p(out))
    return out


def warp_nearest_label(pos, lab, prec=32):
    pos = _f(pos, prec)
    lab = np.ascontiguousarray(lab, dtype=np.int16)
    out = np.empty_like(lab)
    getattr(lib(prec), f"fro{prec}_warp_nearest_label")(_dims(lab.shape), _p(pos), _p(lab), _p(out))
    return out


def ref_register(params, T, labT, S, labS, prec=32, state=None):
    """Full reference-mode registration.  params: fastreg_gb300.Params-like object.
    Returns dict with out_T/out_labT/out_S/out_labS, rho, v, psi, psi_inv, iterations,
    converged, trace_norm, trace_idx."""
    T, S = _f(T, prec), _f(S, prec)
    labT = np.ascontiguousarray(labT, np.int16)
    labS = np.ascontiguousarray(labS, np.int16)
    z, y, x = T.shape
    P = (RefParams32 if prec == 32 else RefParams64)()
    P.max_iter = int(params.max_iter)
    P.reset_iter = int(params.reset_iter)
    P.max_update_norm = params.max_update_norm
    P.rho_0, P.tau, P.w_reg, P.alpha, P.p, P.C = (params.rho_0, params.tau, params.w_reg, params.alpha, params.p,
                                                  params.C)
    dt = _dt(prec)
    if state is not None:
        P.keep_state = 1
        rho = _f(state["rho"], prec).copy()
        v = _f(state["v"], prec).copy()
        psi = _f(state["psi"], prec).copy()
        pinv = _f(state["psi_inv"], prec).copy()
    else:
        P.keep_state = 0
        rho = np.empty((z, y, x), dt)
        v = np.empty((3, z, y, x), dt)
        psi = np.empty((3, z, y, x), dt)
        pinv = np.empty((3, z, y, x), dt)
    oT, oS = np.empty_like(T), np.empty_like(S)
    olT, olS = np.empty_like(labT), np.empty_like(labS)
    n = max(int(params.max_iter), 1)
    tn = np.zeros(n, dt)
    ti = np.zeros(n, np.int64)
    conv = C.c_int()
    ran = getattr(lib(prec), f"fro{prec}_ref_register")(
        _dims(T.shape), C.byref(P), _p(T), _p(labT), _p(S), _p(labS), _p(rho), _p(v), _p(psi), _p(pinv), _p(oT),
        _p(olT), _p(oS), _p(olS), _p(tn), _p(ti), C.byref(conv))
    return dict(out_T=oT, out_labT=olT, out_S=oS, out_labS=olS, rho=rho, v=v, psi=psi, psi_inv=pinv,
                iterations=int(ran), converged=bool(conv.value), trace_norm=tn[:ran], trace_idx=ti[:ran])


def stats(T, labT, warped_S, warped_labS, psi, no_labels, prec=32):
    T, warped_S, psi = _f(T, prec), _f(warped_S, prec), _f(psi, prec)
    labT = np.ascontiguousarray(labT, np.int16)
    warped_labS = np.ascontiguousarray(warped_labS, np.int16)
    st = Stats()
    getattr(lib(prec), f"fro{prec}_stats")(_dims(T.shape), C.c_int(int(no_labels)), _p(T), _p(labT), _p(warped_S),
                                           _p(warped_labS), _p(psi), C.byref(st))
    return dict(e_data=st.e_data, e_reg=st.e_reg, folds=int(st.folds),
                dice_inter=np.array(st.dice_inter[:], np.int64), dice_count=np.array(st.dice_count[:], np.int64),
                dice_out_of_range=int(st.dice_out_of_range))


def deformation_jacobian(psi, prec=32):
    psi = _f(psi, prec)
    z, y, x = psi.shape[1:]
    J = np.empty((9, z, y, x), _dt(prec))
    det = np.empty((z, y, x), _dt(prec))
    getattr(lib(prec), f"fro{prec}_deformation_jacobian")(_dims(psi.shape), _p(psi), _p(J), _p(det))
    return J, det


def ref_det_field(pinv, prec=32):
    pinv = _f(pinv, prec)
    out = np.empty(pinv.shape[1:], _dt(prec))
    getattr(lib(prec), f"fro{prec}_ref_det_field")(_dims(pinv.shape), _p(pinv), _p(out))
    return out


def gaussian_taps(sigma, width, prec=32):
    out = np.empty(width, _dt(prec))
    fn = getattr(lib(prec), f"fro{prec}_gaussian_taps")
    fn.argtypes = [C.c_double, C.c_int, C.c_void_p]
    fn(float(sigma), int(width), _p(out))
    return out


def sob_grad(S, T, phi, lam=0.0, prec=32):
    S, T, phi = _f(S, prec), _f(T, prec), _f(phi, prec)
    g = np.empty_like(phi)
    W = np.empty_like(S)
    real = C.c_float if prec == 32 else C.c_double
    fn = getattr(lib(prec), f"fro{prec}_sob_grad")
    fn.restype = C.c_double
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, real, C.c_void_p, C.c_void_p]
    e = fn(_dims(S.shape), _p(S), _p(T), _p(phi), lam, _p(g), _p(W))
    return g, float(e), W


def sob_smooth3(g, m, sigma, width, damping, step, prec=32):
    """x, y, z passes with the momentum update fused into the z pass; returns new m."""
    g = _f(g, prec).copy()
    m = _f(m, prec).copy()
    taps = gaussian_taps(sigma, width, prec)
    tmp = np.empty_like(g)
    real = C.c_float if prec == 32 else C.c_double
    fn = getattr(lib(prec), f"fro{prec}_sob_smooth")
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, real, real]
    d = _dims(g.shape)
    R = int(width) // 2
    fn(d, _p(taps), R, 0, _p(g), _p(tmp), 0, 0.0, 0.0)
    fn(d, _p(taps), R, 1, _p(tmp), _p(g), 0, 0.0, 0.0)
    fn(d, _p(taps), R, 2, _p(g), _p(m), 1, damping, step)
    return m


def sob_pass_b(m, phi, prec=32):
    m = _f(m, prec)
    phi = _f(phi, prec).copy()
    real = C.c_float if prec == 32 else C.c_double
    mx = real()
    am = C.c_int64()
    getattr(lib(prec), f"fro{prec}_sob_pass_b")(_dims(m.shape), _p(m), _p(phi), C.byref(mx), C.byref(am))
    return phi, float(mx.value), int(am.value)


def sob_register(params, T, S, prec=32):
    T, S = _f(T, prec), _f(S, prec)
    P = (SobParams32 if prec == 32 else SobParams64)()
    P.max_iter = int(params.max_iter)
    P.max_update_norm = params.max_update_norm
    P.damping, P.step, P.sigma, P.width = params.damping, params.step, params.smooth_sigma, int(params.smooth_width)
    P.lam = params.w_reg
    z, y, x = T.shape
    dt = _dt(prec)
    phi = np.empty((3, z, y, x), dt)
    m = np.empty((3, z, y, x), dt)
    n = max(int(params.max_iter), 1)
    tn = np.zeros(n, dt)
    ti = np.zeros(n, np.int64)
    te = np.zeros(n, np.float64)
    conv = C.c_int()
    ran = getattr(lib(prec), f"fro{prec}_sob_register")(_dims(T.shape), C.byref(P), _p(T), _p(S), _p(phi), _p(m),
                                                       _p(tn), _p(ti), _p(te), C.byref(conv))
    return dict(phi=phi, m=m, iterations=int(ran), converged=bool(conv.value), trace_norm=tn[:ran],
                trace_idx=ti[:ran], trace_energy=te[:ran])


def sob_loss_grad(params, T, S, v0, lam, iters, with_grad=True, prec=64):
    """J = 0.5 sum (S(phi_K) - T)^2 + 0.1 sum |m_K|^2 of a K-iteration sobolev
    registration from phi = identity, m = v0; returns (J, dJ/dv0, dJ/dlambda)."""
    T, S, v0 = _f(T, prec), _f(S, prec), _f(v0, prec)
    real = C.c_float if prec == 32 else C.c_double
    P = (SobGradParams32 if prec == 32 else SobGradParams64)()
    P.iters, P.damping, P.step, P.sigma, P.width = int(iters), params.damping, params.step, params.smooth_sigma, \
        int(params.smooth_width)
    fn = getattr(lib(prec), f"fro{prec}_sob_loss_grad")
    fn.restype = C.c_double
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, real, C.c_void_p, C.c_void_p]
    gv = np.zeros_like(v0) if with_grad else None
    gl = C.c_double()
    J = fn(_dims(T.shape), C.byref(P), _p(T), _p(S), _p(v0), lam, _p(gv) if with_grad else None, C.byref(gl))
    return float(J), gv, float(gl.value)


def warp_adjoint(pos, img, wbar, prec=64):
    pos, img, wbar = _f(pos, prec), _f(img, prec), _f(wbar, prec)
    pb = np.empty_like(pos)
    ib = np.empty_like(img)
    getattr(lib(prec), f"fro{prec}_warp_adjoint")(_dims(img.shape), _p(pos), _p(img), _p(wbar), _p(pb), _p(ib))
    return pb, ib


def warp_sob(pos, img, prec=64):
    pos, img = _f(pos, prec), _f(img, prec)
    out = np.empty_like(img)
    getattr(lib(prec), f"fro{prec}_warp_sob")(_dims(img.shape), _p(pos), _p(img), _p(out))
    return out
