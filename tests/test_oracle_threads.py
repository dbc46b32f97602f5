"""The oracle's OpenMP loops do not change any result: a reference-mode and a sobolev
registration, run in child processes with 1 and with 3 threads, give the same bits
(fields, warped images and labels, max-update traces with their voxels, FP64 energies),
and so does the FP64 adjoint of an unrolled sobolev registration."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent

CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from fastreg_gb300 import Params
from oracle import oracle as O
from tests.helpers import images
dims = (23, 19, 17)
d = images(dims, 41)
P = Params(volume_dims=dims, no_labels=4, max_iter=15, alpha=0.02)
o = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"])
Ps = Params(volume_dims=dims, no_labels=4, max_iter=15, solver="sobolev", smooth_sigma=1.5, smooth_width=7,
            damping=0.9, step=0.5)
s = O.sob_register(Ps, d["T"], d["S"])
from tests.helpers import rng, smooth_noise
v0 = smooth_noise(rng(5), (3,) + dims[::-1], 0.3).astype(np.float64)
J, gv, gl = O.sob_loss_grad(Ps, d["T"], d["S"], v0, 0.2, 6)
np.savez(sys.argv[2], adj_J=np.float64(J), adj_gv=gv, adj_gl=np.float64(gl), psi=o["psi"], psi_inv=o["psi_inv"], out_S=o["out_S"], out_labS=o["out_labS"],
         out_T=o["out_T"], tn=o["trace_norm"], ti=o["trace_idx"], phi=s["phi"], m=s["m"], stn=s["trace_norm"],
         sti=s["trace_idx"], ste=s["trace_energy"])
"""


def _run(threads, out):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT), str(out)], env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(out)


def test_oracle_is_independent_of_the_thread_count(tmp_path):
    a = _run(1, tmp_path / "t1.npz")
    b = _run(3, tmp_path / "t3.npz")
    for k in a.files:
        x, y = a[k], b[k]
        assert x.shape == y.shape, k
        assert x.tobytes() == y.tobytes(), f"{k} differs between 1 and 3 OpenMP threads"
