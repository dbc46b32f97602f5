"""Build the CPU oracle (test infrastructure only).

Compiles oracle/fr_oracle.c twice with gcc -- FP32 op-order matched (fro32_*) and
FP64 (fro64_*) -- into oracle/_build/.  -ffp-contract=off keeps a*b+c uncontracted
on every host (gcc contracts by default on aarch64); OpenMP parallelises the
per-voxel loops for the timed CPU baseline without changing any result.
"""
from __future__ import annotations

import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
SRC = HERE / "fr_oracle.c"
FLAGS = ["-O2", "-fPIC", "-shared", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-Wall"]


def build(verbose: bool = False) -> dict:
    OUT.mkdir(exist_ok=True)
    libs = {}
    for tag, defs in (("32", []), ("64", ["-DFRO_DOUBLE", "-DFRO_REAL=double"])):
        out = OUT / f"libfr_oracle{tag}.so"
        tmp = OUT / f"libfr_oracle{tag}.so.tmp"
        cmd = ["gcc", *FLAGS, *defs, "-o", str(tmp), str(SRC), "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stderr}")
        tmp.replace(out)
        libs[tag] = out
        if verbose:
            print(f"built {out}")
    return libs


if __name__ == "__main__":
    build(verbose=True)
