"""The C ABI library without a GPU: it loads, exports every entry point that
include/fastreg_gb300.h declares, parses params.ini like the reference app, and
fails with status codes (never exits) where a GPU would be needed."""
import ctypes as C
import os
import re
import subprocess
from pathlib import Path

import pytest

from fastreg_gb300 import Params, _native as N

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_entry_points():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s*(fr_[a-z0-9_]+)\s*\(", text, re.M):
            names.add(m.group(1))
    return names


def exported_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", str(N.LIB_PATH)], capture_output=True, text=True, check=True)
    return {line.split()[-1] for line in out.stdout.splitlines() if " T " in line}


def test_library_loads_and_exports_every_declared_symbol():
    lib = N.load()
    decl = declared_entry_points()
    assert len(decl) >= 15
    exp = exported_symbols()
    missing = decl - exp
    assert not missing, f"declared in include/*.h but not exported: {sorted(missing)}"
    for name in decl:
        getattr(lib, name)  # resolvable through ctypes
    # everything the ctypes binding wraps is declared
    assert {n for n, _, _ in N.SIGNATURES} <= decl
    assert lib.fr_abi_version() == 3


REFERENCE_INI = """# IMAGES
VOL_DIMS_X=193
VOL_DIMS_Y=229
VOL_DIMS_Z=193

VOL_SIZE_X=1.0
VOL_SIZE_Y=1.0
VOL_SIZE_Z=1.0

NO_LABELS=6

# SOLVER
ALPHA=0.004

MAX_ITER=2048
MAX_UPDATE_NORM=-1e-10

RHO_0=1.0
TAU=0.2
W_REG=0.2

RESET_ITER=-1

p=2.0
C=0.25
"""


def test_params_ini_parses_like_the_reference_app():
    P = Params.from_ini_text(REFERENCE_INI)
    assert P.volume_dims == (193, 229, 193)
    assert P.no_labels == 6 and P.max_iter == 2048 and P.reset_iter == -1
    assert abs(P.alpha - 0.004) < 1e-9 and abs(P.max_update_norm + 1e-10) < 1e-15
    assert P.rho_0 == 1.0 and abs(P.tau - 0.2) < 1e-7 and abs(P.w_reg - 0.2) < 1e-7
    assert P.p == 2.0 and P.C == 0.25 and P.solver == "reference"


def test_params_ini_variant_keys_and_errors(tmp_path):
    P = Params.from_ini_text("SOLVER=sobolev\nSMOOTH_SIGMA=2.0\nSMOOTH_WIDTH=9\nDAMPING=0.8\nSTEP=0.25\n"
                             "KEEP_STATE=1\n[section]\n  MAX_ITER = 7  # comment\n")
    assert P.solver == "sobolev" and P.smooth_sigma == 2.0 and P.smooth_width == 9
    assert abs(P.damping - 0.8) < 1e-7 and P.step == 0.25 and P.keep_state == 1 and P.max_iter == 7
    assert P.autotune == 1  # the default
    assert Params.from_ini_text("AUTOTUNE=0\n").autotune == 0
    assert P.staging == 0 and Params.from_ini_text("STAGING=2\n").staging == 2
    with pytest.raises(N.FastRegError) as e:
        Params.from_ini_text("NOT_A_KEY=1\n")
    assert e.value.status == N.FR_ERR_PARSE and "NOT_A_KEY" in str(e.value)
    with pytest.raises(N.FastRegError) as e:
        Params.from_ini_text("MAX_ITER=abc\n")
    assert e.value.status == N.FR_ERR_PARSE
    with pytest.raises(N.FastRegError) as e:
        Params.from_ini_text("MAX_ITER\n")
    assert e.value.status == N.FR_ERR_PARSE
    with pytest.raises(N.FastRegError) as e:
        Params.from_ini(str(tmp_path / "missing.ini"))
    assert e.value.status == N.FR_ERR_IO
    f = tmp_path / "p.ini"
    f.write_text(REFERENCE_INI)
    assert Params.from_ini(str(f)).volume_dims == (193, 229, 193)


def test_invalid_params_are_rejected_with_status():
    lib = N.load()
    h = C.c_void_p()
    for bad in (dict(no_labels=0), dict(no_labels=300), dict(max_iter=-1), dict(alpha=0.0),
                dict(solver="sobolev", smooth_width=8), dict(verbosity=5), dict(staging=3)):
        P = Params(**bad)
        c = P.to_c()
        if "solver" in bad:
            c.solver = N.FR_SOLVER_SOBOLEV
        rc = lib.fr_create(C.byref(c), C.byref(h))
        assert rc == N.FR_ERR_INVALID_ARG, bad
        assert h.value is None
    assert lib.fr_create(None, C.byref(h)) != N.FR_OK


def test_no_gpu_gives_a_status_not_an_exit():
    """fr_create on a machine without a usable GPU returns FR_ERR_CUDA (the reference
    would print and exit(0), device_memory.cpp:10-13)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = N.load()
    h = C.c_void_p()
    rc = lib.fr_create(C.byref(Params(volume_dims=(8, 8, 8)).to_c()), C.byref(h))
    assert rc == N.FR_ERR_CUDA
    assert b"CUDA" in lib.fr_last_error(None) or len(lib.fr_last_error(None)) > 0
    assert lib.fr_status_string(N.FR_ERR_CUDA) == b"CUDA error"
    dims = (C.c_int * 3)(8, 8, 8)
    assert lib.fr_warp(None, None, None, dims, None, None, None) == N.FR_ERR_INVALID_ARG


CPP_CALLER = r'''
#include <cstdio>
#include "fastreg_compat.hpp"

int main(int argc, char** argv) {
    Params params = Params::from_ini(argv[1]);
    std::printf("dims %d %d %d alpha %g iters %d\n", params.volume_dims[0], params.volume_dims[1],
                params.volume_dims[2], params.alpha, params.max_iter);
    try {
        FastReg fastreg(params);
        std::printf("created\n");
    } catch (const fastreg_gb300::Error& e) {
        std::printf("error %d\n", e.status);
    }
    return 0;
}
'''


def test_cpp_shim_compiles_and_runs(tmp_path):
    """A demo.cpp-style caller compiles against include/fastreg_compat.hpp (the
    reference's Params/FastReg names) and runs; without a GPU, FastReg's
    constructor throws fastreg_gb300::Error(FR_ERR_CUDA) instead of exiting."""
    import shutil
    import torch
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "caller.cpp"
    src.write_text(CPP_CALLER)
    ini = tmp_path / "params.ini"
    ini.write_text(REFERENCE_INI)
    exe = tmp_path / "caller"
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    cmd = ["g++", "-std=c++17", "-O1", str(src), "-o", str(exe), "-I", str(ROOT / "include"), "-I",
           str(cuda / "include"), "-L", str(N.LIB_PATH.parent), "-lfastreg_gb300", "-L", str(cuda / "lib64"),
           "-lcudart", f"-Wl,-rpath,{N.LIB_PATH.parent}", f"-Wl,-rpath,{cuda / 'lib64'}"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe), str(ini)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert "dims 193 229 193" in out.stdout and "iters 2048" in out.stdout
    if not torch.cuda.is_available():
        assert f"error {N.FR_ERR_CUDA}" in out.stdout
    else:
        assert "created" in out.stdout


LIMITS_CHECK = r'''
#include <cstdio>
#include <initializer_list>
#include "fr_limits.h"
int main() {
    const long long M = frg::kIndex32Max;
    int bad = 0;
    auto want = [&](long long X, long long Y, long long Z, bool ok) {
        if (frg::fits_index32(X, Y, Z) != ok) { std::printf("wrong: %lld %lld %lld\n", X, Y, Z); ++bad; }
    };
    // the largest volume of pitch X and Y rows whose far-corner and prefetch offsets fit
    for (long long X : {4LL, 184LL, 1024LL, 2048LL})
        for (long long Y : {1LL, 218LL, 1024LL}) {
            const long long XY = X * Y, Zmax = (M - 2 * XY - 2 * X - 2) / XY;
            want(X, Y, Zmax, true);
            want(X, Y, Zmax + 1, false);
        }
    want(184, 218, 182, true);
    want(0, 5, 5, false);
    want(1LL << 20, 1LL << 20, 1LL << 20, false);   // X*Y*Z overflows 64-bit arithmetic checks
    want(46341, 46341, 1, false);                   // X*Y alone above 2^31 - 1
    std::printf(bad ? "FAIL\n" : "OK\n");
    return bad;
}
'''


def test_index32_predicate(tmp_path):
    """The 32-bit kernels take a volume only when its largest corner and prefetch
    offset (N + 2 X Y + 2 X + 2) fits an int: the predicate at its boundary."""
    import shutil
    if shutil.which("g++") is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "limits.cpp"
    src.write_text(LIMITS_CHECK)
    exe = tmp_path / "limits"
    subprocess.run(["g++", "-std=c++17", "-O1", str(src), "-o", str(exe), "-I",
                    str(ROOT / "fastreg_gb300" / "csrc")], check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and "OK" in out.stdout, out.stdout

