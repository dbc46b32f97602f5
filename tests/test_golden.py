"""The CPU oracle against the golden outputs of the reference's own CUDA kernels.

The fixtures under tests/golden were produced by tests/golden/make_golden.py, which
runs the reference's unmodified kernels (compiled from its sources, launched in its
order by oracle/ref_runner.c) on a GB300.  The reference build uses --ftz=true,
--prec-div=false, --prec-sqrt=false and nvcc's default FMA contraction, so it is
compared within tolerances, not bit for bit:
  - positions psi / psi_inv: |oracle - reference| <= 1e-5 * max(1, |reference|);
  - warped intensities: <= 1e-5 relative (floor 1e-6 absolute);
  - max-update-norm trace: <= 1e-4 relative;
  - floor-corner labels: identical wherever the sample position is farther than
    1e-4 voxel from an integer grid plane (where the floor itself is decided by
    the last bits of psi).
"""
from pathlib import Path

import numpy as np
import pytest

from fastreg_gb300 import Params
from oracle import oracle as O

GOLDEN = sorted(Path(__file__).resolve().parent.joinpath("golden").glob("ref_*.npz"))


def _params(f):
    dims = tuple(int(v) for v in f["dims"])
    pv = f["params"]
    return Params(volume_dims=dims, no_labels=4, max_iter=int(pv[0]), reset_iter=int(pv[1]),
                  max_update_norm=float(pv[2]), rho_0=float(pv[3]), tau=float(pv[4]), w_reg=float(pv[5]),
                  alpha=float(pv[6]), p=float(pv[7]), C=float(pv[8]))


def _near_grid(pos, eps=1e-4):
    c = np.clip(pos, 0, None)
    return (np.abs(c - np.round(c)) < eps).any(axis=0)


@pytest.mark.skipif(not GOLDEN, reason="no golden fixtures")
@pytest.mark.parametrize("path", GOLDEN, ids=[p.stem for p in GOLDEN])
def test_oracle_matches_reference_kernels(path):
    f = np.load(path)
    P = _params(f)
    o = O.ref_register(P, f["T"], f["labT"], f["S"], f["labS"])
    assert o["iterations"] == int(f["iterations"])
    for k in ("psi", "psi_inv"):
        ref = f[k].astype(np.float64)
        err = np.abs(o[k] - ref) / np.maximum(1.0, np.abs(ref))
        assert err.max() <= 1e-5, f"{k}: max error {err.max():.3g}"
    for k in ("out_T", "out_S"):
        ref = f[k].astype(np.float64)
        err = np.abs(o[k] - ref) / np.maximum(1e-1, np.abs(ref))
        assert err.max() <= 1e-5, f"{k}: max error {err.max():.3g}"
    tn = f["trace_norm"].astype(np.float64)
    err = np.abs(o["trace_norm"] - tn) / np.maximum(tn, 1e-12)
    assert err.max() <= 1e-4, f"max-norm trace: {err.max():.3g}"
    for lab, pos in (("out_labS", o["psi"]), ("out_labT", o["psi_inv"])):
        diff = o[lab] != f[lab]
        assert not (diff & ~_near_grid(pos)).any(), f"{lab}: {int(diff.sum())} labels differ away from grid planes"
