"""Build the reference's own CUDA kernels as cubins (test infrastructure only).

The five unmodified translation units src/fastreg/cuda/{solver,vector_fields,
reductor,scalar_fields,volume}.cu of the reference are compiled where they lie
(read-only; the tree named by the FASTREG_REFERENCE environment variable, by
default the directory `reference` beside this repository) with the reference's own
nvcc flags
(CMakeLists.txt:39-46: --ftz=true --prec-div=false --prec-sqrt=false
--expt-relaxed-constexpr), retargeted to sm_103a, into oracle/_ref/*.cubin.  Only
device code is built: the host side of the reference loop (estimate_psi,
solver.cu:295-444) is driven by oracle/ref_runner.c through the CUDA driver API.
The one OpenCV type the headers need comes from oracle/ref_shim.

Nothing here runs where the reference sources are absent (the GPU machine): the
cubins built here travel in oracle/_ref/.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
REF = Path(os.environ.get("FASTREG_REFERENCE", str(HERE.parent.parent / "reference")))
OUT = HERE / "_ref"
UNITS = ("solver", "vector_fields", "reductor", "scalar_fields", "volume")
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "--ftz=true", "--prec-div=false", "--prec-sqrt=false",
         "--expt-relaxed-constexpr", "-std=c++14", "-O3"]


def available() -> bool:
    return (REF / "src" / "fastreg" / "cuda" / "solver.cu").exists()


def build_if_available(verbose: bool = False) -> bool:
    """Build the cubins when the reference tree is present; returns whether the
    cubins exist afterwards."""
    if available():
        OUT.mkdir(exist_ok=True)
        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        for u in UNITS:
            src = REF / "src" / "fastreg" / "cuda" / f"{u}.cu"
            out = OUT / f"{u}.cubin"
            cmd = [nvcc, *FLAGS, "-I", str(REF / "include"), "-I", str(HERE / "ref_shim"), "-cubin", str(src),
                   "-o", str(out)]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"reference kernel build failed on {u}.cu:\n{r.stderr}")
            if verbose:
                print(f"built {out}")
    have = all((OUT / f"{u}.cubin").exists() for u in UNITS)
    if have:
        build_runner(verbose)
    return have


def build_runner(verbose: bool = False) -> Path:
    """The driver-API host of the reference loop (compiled on every machine)."""
    OUT.mkdir(exist_ok=True)
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    out = OUT / "libref_runner.so"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-std=c11", "-Wall", "-I", str(cuda / "include"),
           str(HERE / "ref_runner.c"), "-o", str(out), "-L", str(cuda / "lib64"), "-L", str(cuda / "lib64" / "stubs"),
           "-lcuda", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ref_runner build failed:\n{r.stderr}")
    if verbose:
        print(f"built {out}")
    return out


if __name__ == "__main__":
    print("cubins:", build_if_available(verbose=True))
