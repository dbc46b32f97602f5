"""Per-pair regularisation weights tuned by hypergradients, then one batched registration.

For each pair the weight lambda (W_REG of the sobolev solver) takes a few steps of
descent on J(lambda) = 0.5 sum (S o phi_K - T)^2 + 0.1 sum |m_K|^2 of a short unrolled
registration, whose dJ/dlambda comes from the hand-written adjoint kernels
(fr_sobolev_loss_grad, forward states checkpointed).  The cohort is then registered in
one fr_register_batch with each pair's own weight (fr_set_pair_w_reg).
"""
from __future__ import annotations

import ctypes as C
import math

from . import _native as N


def sobolev_loss_grad(T, S, params, w_reg: float, iters: int, checkpoint_every: int = 10, v0=None, stream=None):
    """J and dJ/dlambda (and dJ/dv0) of an `iters`-iteration sobolev registration of
    S to T (CUDA float32 tensors (Z, Y, X)) from momentum v0 (zeros by default)."""
    import torch
    lib = N.load()
    z, y, x = T.shape
    if v0 is None:
        v0 = torch.zeros((3, z, y, x), device=T.device, dtype=torch.float32)
    gv = torch.empty_like(v0)
    dims = (C.c_int * 3)(x, y, z)
    loss, gl = C.c_double(), C.c_double()
    s = None if stream is None else stream.cuda_stream
    N.check(lib.fr_sobolev_loss_grad(T.data_ptr(), S.data_ptr(), dims, v0.data_ptr(), float(w_reg), int(iters),
                                     int(checkpoint_every), params.damping, params.step, params.smooth_sigma,
                                     int(params.smooth_width), C.byref(loss), gv.data_ptr(), C.byref(gl), s),
            None, "fr_sobolev_loss_grad")
    return loss.value, gl.value, gv


def tune_w_reg(T, S, params, w0: float | None = None, steps: int = 5, iters: int = 30, checkpoint_every: int = 10,
               rate: float = 0.5, stream=None):
    """`steps` hypergradient steps on log(lambda): the step is -rate * tanh(e), e the
    elasticity lambda * dJ/dlambda / J, so each step changes lambda by a factor within
    [exp(-rate), exp(rate)].  Returns the final lambda and the (lambda, J, dJ/dlambda)
    history."""
    lam = float(params.w_reg if w0 is None else w0)
    hist = []
    for _ in range(steps):
        J, g, _ = sobolev_loss_grad(T, S, params, lam, iters, checkpoint_every, stream=stream)
        hist.append((lam, J, g))
        e = lam * g / max(abs(J), 1e-30)
        lam = lam * math.exp(-rate * math.tanh(e))
    return lam, hist


def register_cohort_tuned(fr, pairs, params, steps: int = 5, iters: int = 30, checkpoint_every: int = 10,
                          stream=None):
    """Tune each pair's weight (tune_w_reg on the pair's (T, S)), then register the cohort
    in one batched call with those weights.  pairs: (img_T, lab_T, img_S, lab_S) CUDA
    tensors, overwritten in place by the registration.  Returns the weights."""
    weights = []
    for (iT, _, iS, _) in pairs:
        lam, _ = tune_w_reg(iT, iS, params, steps=steps, iters=iters, checkpoint_every=checkpoint_every,
                            stream=stream)
        weights.append(lam)
    fr.set_pair_w_reg(weights)
    fr.register_batch(pairs, stream=stream)
    return weights
