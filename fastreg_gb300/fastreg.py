"""Host-side mirror of the reference's public interface: ``Params`` (include/params.hpp)
and ``FastReg`` (include/fastreg.hpp, src/fastreg/fastreg.cpp), over the C ABI.

Volumes are CUDA tensors of shape (Z, Y, X), x fastest, exactly the reference's
linear layout; vector fields are (3, Z, Y, X).  ``FastReg.__call__`` overwrites
its four arguments in place like ``FastReg::operator()``: the target buffers
receive T o psi_inv, the source buffers S o psi.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field, fields
from typing import Sequence

from . import _native as N


@dataclass
class Params:
    """struct Params (include/params.hpp:7-26) plus the sobolev solver keys."""
    volume_dims: tuple = (193, 229, 193)
    volume_size: tuple = (1.0, 1.0, 1.0)
    no_labels: int = 6
    max_iter: int = 2048
    max_update_norm: float = -1e-10
    rho_0: float = 1.0
    tau: float = 0.2
    w_reg: float = 0.2
    alpha: float = 0.004
    p: float = 2.0
    C: float = 0.25
    reset_iter: int = -1
    verbosity: int = 0
    solver: str = "reference"
    smooth_sigma: float = 1.5
    smooth_width: int = 7
    damping: float = 0.9
    step: float = 0.5
    keep_state: int = 0
    autotune: int = 1
    staging: int = 0

    @classmethod
    def from_c(cls, c: N.fr_params) -> "Params":
        return cls(
            volume_dims=tuple(c.volume_dims), volume_size=tuple(c.volume_size), no_labels=c.no_labels,
            max_iter=c.max_iter, max_update_norm=c.max_update_norm, rho_0=c.rho_0, tau=c.tau, w_reg=c.w_reg,
            alpha=c.alpha, p=c.p, C=c.C, reset_iter=c.reset_iter, verbosity=c.verbosity,
            solver="sobolev" if c.solver == N.FR_SOLVER_SOBOLEV else "reference",
            smooth_sigma=c.smooth_sigma, smooth_width=c.smooth_width, damping=c.damping, step=c.step,
            keep_state=c.keep_state, autotune=c.autotune, staging=c.staging)

    def to_c(self) -> N.fr_params:
        c = N.fr_params()
        c.volume_dims[:] = [int(v) for v in self.volume_dims]
        c.volume_size[:] = [float(v) for v in self.volume_size]
        c.no_labels = int(self.no_labels)
        c.max_iter = int(self.max_iter)
        c.max_update_norm = float(self.max_update_norm)
        c.rho_0 = float(self.rho_0)
        c.tau = float(self.tau)
        c.w_reg = float(self.w_reg)
        c.alpha = float(self.alpha)
        c.p = float(self.p)
        c.C = float(self.C)
        c.reset_iter = int(self.reset_iter)
        c.verbosity = int(self.verbosity)
        c.solver = N.FR_SOLVER_SOBOLEV if self.solver == "sobolev" else N.FR_SOLVER_REFERENCE
        c.smooth_sigma = float(self.smooth_sigma)
        c.smooth_width = int(self.smooth_width)
        c.damping = float(self.damping)
        c.step = float(self.step)
        c.keep_state = int(self.keep_state)
        c.autotune = int(self.autotune)
        c.staging = int(self.staging)
        return c

    @classmethod
    def from_ini_text(cls, text: str) -> "Params":
        lib = N.load()
        c = N.fr_params()
        N.check(lib.fr_params_default(C.byref(c)))
        N.check(lib.fr_params_parse_ini(text.encode(), C.byref(c)), None, "params.ini")
        return cls.from_c(c)

    @classmethod
    def from_ini(cls, path: str) -> "Params":
        lib = N.load()
        c = N.fr_params()
        N.check(lib.fr_params_default(C.byref(c)))
        N.check(lib.fr_params_load_ini(str(path).encode(), C.byref(c)), None, str(path))
        return cls.from_c(c)

    def no_voxels(self) -> int:
        x, y, z = self.volume_dims
        return int(x) * int(y) * int(z)


def _ptr(t) -> int:
    """Device address of a CUDA tensor (or an int address)."""
    if isinstance(t, int):
        return t
    if not t.is_cuda:
        raise ValueError("fastreg_gb300 works on CUDA device buffers")
    if not t.is_contiguous():
        raise ValueError("buffers must be contiguous")
    return t.data_ptr()


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


@dataclass
class Stats:
    iterations: int
    converged: bool
    last_max_update_norm: float
    last_max_update_voxel: int
    e_data: float
    e_reg: float
    energy: float
    folds: int
    dice: list = field(default_factory=list)
    dice_all: float = float("nan")
    dice_out_of_range: int = 0
    dice_inter: list = field(default_factory=list)
    dice_count: list = field(default_factory=list)


class FastReg:
    """FastReg (include/fastreg.hpp:12-38) backed by the GB300 kernels."""

    def __init__(self, params: Params):
        self.lib = N.load()
        self.params = params
        self._c = params.to_c()
        h = C.c_void_p()
        N.check(self.lib.fr_create(C.byref(self._c), C.byref(h)), None, "fr_create")
        self.h = h
        self.frame_counter = 0
        self._dims = [tuple(int(v) for v in params.volume_dims)]

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.fr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self) -> Params:
        return self.params

    # FastReg::operator() -- enqueues on `stream`; synchronizes unless sync=False
    def __call__(self, img_T, lab_T, img_S, lab_S, stream=None, sync: bool = True) -> bool:
        self._check_shape(img_T, lab_T, img_S, lab_S, self.params.volume_dims)
        st = _stream_ptr(stream)
        self._dims = [tuple(int(v) for v in self.params.volume_dims)]
        N.check(self.lib.fr_register(self.h, _ptr(img_T), _ptr(lab_T), _ptr(img_S), _ptr(lab_S), st), self.h,
                "fr_register")
        if sync:
            self._sync(stream)
        self.frame_counter += 1
        return True

    def register_batch(self, pairs: Sequence[tuple], stream=None, sync: bool = True) -> None:
        """pairs: sequence of (img_T, lab_T, img_S, lab_S) CUDA tensors of shape (Z, Y, X)."""
        arr = (N.fr_pair * len(pairs))()
        for k, (iT, lT, iS, lS) in enumerate(pairs):
            z, y, x = iT.shape
            self._check_shape(iT, lT, iS, lS, (x, y, z))
            arr[k].dims[:] = [x, y, z]
            arr[k].img_T, arr[k].lab_T, arr[k].img_S, arr[k].lab_S = _ptr(iT), _ptr(lT), _ptr(iS), _ptr(lS)
        self._dims = [tuple(arr[k].dims) for k in range(len(pairs))]
        N.check(self.lib.fr_register_batch(self.h, arr, len(pairs), _stream_ptr(stream)), self.h,
                "fr_register_batch")
        if sync:
            self._sync(stream)

    # the phases, for stepping the solver from an arbitrary state
    def begin(self, pairs: Sequence[tuple], stream=None) -> None:
        arr = (N.fr_pair * len(pairs))()
        for k, (iT, lT, iS, lS) in enumerate(pairs):
            z, y, x = iT.shape
            arr[k].dims[:] = [x, y, z]
            arr[k].img_T, arr[k].lab_T, arr[k].img_S, arr[k].lab_S = _ptr(iT), _ptr(lT), _ptr(iS), _ptr(lS)
        self._dims = [tuple(arr[k].dims) for k in range(len(pairs))]
        N.check(self.lib.fr_begin(self.h, arr, len(pairs), _stream_ptr(stream)), self.h, "fr_begin")

    def step(self, it: int, t: float, stream=None) -> None:
        N.check(self.lib.fr_step(self.h, int(it), float(t), _stream_ptr(stream)), self.h, "fr_step")

    def finish(self, stream=None) -> None:
        N.check(self.lib.fr_finish(self.h, _stream_ptr(stream)), self.h, "fr_finish")

    def get_field(self, which: int, pair: int = 0, out=None, stream=None):
        import torch
        dims = self._pair_dims(pair, out)
        x, y, z = dims
        ncomp = 1 if which == N.FR_FIELD_RHO else 3
        if out is None:
            out = torch.empty((ncomp, z, y, x) if ncomp == 3 else (z, y, x), dtype=torch.float32, device="cuda")
        N.check(self.lib.fr_get_field(self.h, pair, which, _ptr(out), _stream_ptr(stream)), self.h, "fr_get_field")
        torch.cuda.synchronize()
        return out

    def set_field(self, which: int, buf, pair: int = 0, stream=None) -> None:
        import torch
        N.check(self.lib.fr_set_field(self.h, pair, which, _ptr(buf), _stream_ptr(stream)), self.h, "fr_set_field")
        torch.cuda.synchronize()

    def get_deformation_field(self, pair: int = 0):
        """FastReg::getDeformationField(): psi as a (3, Z, Y, X) CUDA tensor."""
        return self.get_field(N.FR_FIELD_PSI, pair)

    def stats(self, pair: int = 0) -> Stats:
        s = N.fr_stats()
        N.check(self.lib.fr_get_stats(self.h, pair, C.byref(s)), self.h, "fr_get_stats")
        nl = s.no_labels
        return Stats(
            iterations=s.iterations, converged=bool(s.converged), last_max_update_norm=s.last_max_update_norm,
            last_max_update_voxel=s.last_max_update_voxel, e_data=s.e_data, e_reg=s.e_reg, energy=s.energy,
            folds=s.folds, dice=list(s.dice[:nl]), dice_all=s.dice_all, dice_out_of_range=s.dice_out_of_range,
            dice_inter=list(s.dice_inter[:nl]), dice_count=list(s.dice_count[:nl]))

    def trace(self, pair: int = 0, cap: int | None = None):
        """Max update norm and its voxel for every iteration run."""
        import numpy as np
        cap = cap or max(int(self.params.max_iter), 1)
        norms = np.zeros(cap, np.float32)
        vox = np.zeros(cap, np.int64)
        n = C.c_int()
        N.check(self.lib.fr_get_trace(self.h, pair, norms.ctypes.data, vox.ctypes.data, cap, C.byref(n)), self.h,
                "fr_get_trace")
        m = min(n.value, cap)
        return norms[:m], vox[:m]

    def set_pair_w_reg(self, weights=None) -> None:
        """Per-pair W_REG for the next cohorts (one weight per pair, in order); None goes
        back to params.w_reg."""
        if weights is None:
            N.check(self.lib.fr_set_pair_w_reg(self.h, None, 0), self.h, "fr_set_pair_w_reg")
            return
        w = (C.c_float * len(weights))(*[float(v) for v in weights])
        N.check(self.lib.fr_set_pair_w_reg(self.h, w, len(weights)), self.h, "fr_set_pair_w_reg")

    def tile_shapes(self):
        """(slices per tile, blocks per SM) of the active solver's three kernels, in launch
        order: the defaults or the autotuner's choice for this cohort."""
        out = []
        for k in range(3):
            d, b = C.c_int(), C.c_int()
            N.check(self.lib.fr_tile_shape(self.h, k, C.byref(d), C.byref(b)), self.h, "fr_tile_shape")
            out.append((d.value, b.value))
        return out

    def tile_staging(self):
        """Per kernel of the active solver, in launch order: "tma" when it stages its
        operands with tensor copies, "cp.async" otherwise."""
        out = []
        for k in range(3):
            v = C.c_int()
            N.check(self.lib.fr_tile_staging(self.h, k, C.byref(v)), self.h, "fr_tile_staging")
            out.append("tma" if v.value else "cp.async")
        return out

    # helpers
    def _pair_dims(self, pair, out):
        if out is not None:
            return (out.shape[-1], out.shape[-2], out.shape[-3])
        return tuple(self._dims[pair])

    @staticmethod
    def _check_shape(iT, lT, iS, lS, dims):
        x, y, z = (int(v) for v in dims)
        for name, t in (("img_T", iT), ("lab_T", lT), ("img_S", iS), ("lab_S", lS)):
            if hasattr(t, "shape") and tuple(t.shape) != (z, y, x):
                raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {(z, y, x)}")

    @staticmethod
    def _sync(stream):
        import torch
        if stream is None:
            torch.cuda.synchronize()
        else:
            stream.synchronize()


def warp(pos, img, lab=None, stream=None, out=None, out_lab=None):
    """apply (vector_fields.cu:81-107): img o pos with trilinear intensities and the
    floor-corner label.  pos: (3, Z, Y, X) positions; img: (Z, Y, X)."""
    import torch
    lib = N.load()
    z, y, x = img.shape
    if tuple(pos.shape) != (3, z, y, x):
        raise ValueError("pos must be (3, Z, Y, X)")
    if out is None:
        out = torch.empty_like(img)
    if lab is not None and out_lab is None:
        out_lab = torch.empty_like(lab)
    dims = (C.c_int * 3)(x, y, z)
    N.check(lib.fr_warp(_ptr(pos), _ptr(img), _ptr(lab) if lab is not None else None, dims, _ptr(out),
                        _ptr(out_lab) if out_lab is not None else None, _stream_ptr(stream)), None, "fr_warp")
    return (out, out_lab) if lab is not None else out


def estimate_inverse(psi, psi_inv, sweeps=48, stream=None):
    """DeformationField::get_inverse (vector_fields.cpp:96-103, vector_fields.cu:109-136):
    `sweeps` passes of psi_inv <- -(psi o psi_inv), psi_inv (3, Z, Y, X) updated in place
    and returned."""
    lib = N.load()
    if tuple(psi.shape) != tuple(psi_inv.shape) or psi.dim() != 4 or psi.shape[0] != 3:
        raise ValueError("psi and psi_inv must both be (3, Z, Y, X)")
    _, z, y, x = psi.shape
    dims = (C.c_int * 3)(x, y, z)
    N.check(lib.fr_estimate_inverse(_ptr(psi), _ptr(psi_inv), dims, int(sweeps), _stream_ptr(stream)), None,
            "fr_estimate_inverse")
    return psi_inv


def interpolate_field(field, pos, out=None, stream=None):
    """interpolate_gradient (vector_fields.cu:194-225): a (3, Z, Y, X) field sampled at
    the positions pos (3, Z, Y, X)."""
    import torch
    lib = N.load()
    if tuple(field.shape) != tuple(pos.shape) or field.dim() != 4 or field.shape[0] != 3:
        raise ValueError("field and pos must both be (3, Z, Y, X)")
    if out is None:
        out = torch.empty_like(field)
    _, z, y, x = field.shape
    dims = (C.c_int * 3)(x, y, z)
    N.check(lib.fr_interpolate_field(_ptr(field), _ptr(pos), dims, _ptr(out), _stream_ptr(stream)), None,
            "fr_interpolate_field")
    return out
