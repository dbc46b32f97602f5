"""fastreg_gb300: fastreg's registration inner loop as hand-written CUDA for GB300 (sm_103a).

The product is the C ABI in include/fastreg_gb300.h, implemented by the
in-tree library fastreg_gb300/_lib/libfastreg_gb300.so; this package is its
Python mirror of the reference's Params / FastReg interface.
"""
from .fastreg import FastReg, Params, Stats, estimate_inverse, interpolate_field, warp  # noqa: F401
from . import _native  # noqa: F401

__all__ = ["FastReg", "Params", "Stats", "estimate_inverse", "interpolate_field", "warp"]
