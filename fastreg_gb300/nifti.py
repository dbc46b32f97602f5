"""NIfTI-1 (single-file .nii) read/write for numpy volumes of shape (Z, Y, X), the layout
the command-line app (fastreg_gb300/app) reads and writes."""
from __future__ import annotations

import struct

import numpy as np

_DT = {2: np.uint8, 4: np.int16, 8: np.int32, 16: np.float32, 64: np.float64, 512: np.uint16}
_CODE = {np.dtype(np.float32): 16, np.dtype(np.int16): 4, np.dtype(np.uint8): 2, np.dtype(np.int32): 8,
         np.dtype(np.float64): 64, np.dtype(np.uint16): 512}


def write(path, vol: np.ndarray, pixdim=(1.0, 1.0, 1.0)) -> None:
    vol = np.ascontiguousarray(vol)
    z, y, x = vol.shape
    h = bytearray(348)
    struct.pack_into("<i", h, 0, 348)
    struct.pack_into("<8h", h, 40, 3, x, y, z, 1, 1, 1, 1)
    struct.pack_into("<hh", h, 70, _CODE[vol.dtype], vol.dtype.itemsize * 8)
    struct.pack_into("<8f", h, 76, 1.0, *pixdim, 1.0, 1.0, 1.0, 1.0)
    struct.pack_into("<f", h, 108, 352.0)
    struct.pack_into("<f", h, 112, 0.0)
    struct.pack_into("<4s", h, 344, b"n+1\0")
    with open(path, "wb") as f:
        f.write(bytes(h))
        f.write(b"\0\0\0\0")
        f.write(vol.astype(vol.dtype.newbyteorder("<")).tobytes())


def read(path) -> np.ndarray:
    with open(path, "rb") as f:
        raw = f.read()
    endian = "<" if struct.unpack_from("<i", raw, 0)[0] == 348 else ">"
    if struct.unpack_from(endian + "i", raw, 0)[0] != 348:
        raise ValueError(f"{path} is not a NIfTI-1 file")
    dim = struct.unpack_from(endian + "8h", raw, 40)
    code = struct.unpack_from(endian + "h", raw, 70)[0]
    off = int(struct.unpack_from(endian + "f", raw, 108)[0])
    x, y, z = dim[1], dim[2], dim[3]
    dt = np.dtype(_DT[code]).newbyteorder(endian)
    return np.frombuffer(raw, dtype=dt, count=x * y * z, offset=off).reshape(z, y, x).astype(_DT[code])
