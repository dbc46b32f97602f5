"""Build the native library of fastreg_gb300 in-tree.

nvcc compiles every ``csrc/*.cu`` translation unit for sm_103a in parallel and
links them into ``fastreg_gb300/_lib/libfastreg_gb300.so`` (CUDA runtime linked
statically, no torch dependency).  ``--fmad=false`` is part of the arithmetic
contract: the kernels contract no a*b+c on their own; the fused multiply-adds
they need are written out as fmaf().  It is given to ptxas as well
(``-Xptxas --fmad=false``): the front end's flag alone does not stop ptxas from
fusing a packed f32x2 multiply and add, even ones written with ``.rn``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
OBJDIR = PKG / "_build"
LIBNAME = "libfastreg_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "--fmad=false", "-Xptxas", "--fmad=false", "-std=c++17",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
    "--expt-relaxed-constexpr",
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fastreg_gb300")
    return cand


def _compile(src: Path, extra: list[str]) -> Path:
    obj = OBJDIR / (src.stem + ".o")
    cmd = [nvcc(), *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile and link; returns the path of the shared library."""
    extra = list(extra or [])
    OBJDIR.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu"))
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    out = LIBDIR / LIBNAME
    tmp = LIBDIR / (LIBNAME + ".tmp")
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    if verbose:
        print(f"built {out}")
    build_app(verbose)
    return out


def build_app(verbose: bool = False) -> Path:
    """The command-line app (fastreg_gb300/app), linked against the library."""
    src = PKG / "app" / "fastreg_app.cpp"
    exe = LIBDIR / "fastreg_app"
    cmd = [nvcc(), "-std=c++17", "-O2", str(src), "-o", str(exe), "-L", str(LIBDIR), "-lfastreg_gb300",
           "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"app build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {exe}")
    return exe


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
