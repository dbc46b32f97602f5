"""Generate the golden fixtures that pin the CPU oracle to the reference.

Runs the reference's own CUDA kernels -- compiled from the reference sources into
oracle/_ref/*.cubin by oracle/ref_build.py and launched in the reference's order by
oracle/ref_runner.c -- on seeded synthetic pairs, and stores inputs, parameters and
outputs as compressed .npz files.  Needs a GPU; run from the repository root:

    python tests/golden/make_golden.py [out_dir]      (default: tests/golden)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from fastreg_gb300 import Params, synthetic as sy  # noqa: E402
from oracle import ref_runner  # noqa: E402

# name: (dims, seed, solver parameters)
CASES = {
    "ref_24x20x18_a0.02_it40": ((24, 20, 18), 101, dict(max_iter=40, alpha=0.02)),
    "ref_33x17x20_a0.05_it25_reset7": ((33, 17, 20), 102, dict(max_iter=25, alpha=0.05, reset_iter=7)),
    "ref_32x28x24_paramsini_it200": ((32, 28, 24), 103, dict(max_iter=200, alpha=0.004)),
    "ref_20x18x16_a0.02_converge": ((20, 18, 16), 104, dict(max_iter=60, alpha=0.02, max_update_norm=2e-3)),
}


def case_params(dims, kw):
    base = dict(volume_dims=dims, no_labels=4, max_iter=40, alpha=0.004, tau=0.2, w_reg=0.2, rho_0=1.0, p=2.0,
                C=0.25, reset_iter=-1, max_update_norm=-1e-10)
    base.update(kw)
    return Params(**base)


def case_inputs(dims, seed):
    spec = sy.PairSpec(dims=dims, n_blobs=max(4, dims[0] * dims[1] * dims[2] // 3000), vel_sigma=2.0,
                       max_disp=2.0, n_classes=4, seed=seed)
    return sy.make_pair(spec)


def main(out_dir: Path):
    if not ref_runner.available():
        raise SystemExit("reference cubins missing: build them with oracle/ref_build.py where the reference "
                         "sources are present")
    out_dir.mkdir(parents=True, exist_ok=True)
    for name, (dims, seed, kw) in CASES.items():
        P = case_params(dims, kw)
        d = case_inputs(dims, seed)
        r = ref_runner.register(P, d["T"], d["labT"], d["S"], d["labS"])
        pv = np.array([P.max_iter, P.reset_iter, P.max_update_norm, P.rho_0, P.tau, P.w_reg, P.alpha, P.p, P.C],
                      np.float64)
        np.savez_compressed(out_dir / f"{name}.npz", dims=np.array(dims), params=pv, T=d["T"], labT=d["labT"],
                            S=d["S"], labS=d["labS"], **{k: v for k, v in r.items() if k != "iterations"},
                            iterations=np.array(r["iterations"]))
        print(f"{name}: {r['iterations']} iterations, last max update norm {r['trace_norm'][-1]:.6g}")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else ROOT / "tests" / "golden")
