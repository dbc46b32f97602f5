"""Generate the golden fixtures that pin the CPU oracle to the reference.

Runs the reference's own CUDA kernels -- compiled from the reference sources into
oracle/_ref/*.cubin by oracle/ref_build.py and launched in the reference's order by
oracle/ref_runner.c -- on seeded synthetic pairs, and stores inputs, parameters and
outputs as compressed .npz files.  Needs a GPU; run from the repository root:

    python tests/golden/make_golden.py [out_dir]      (default: tests/golden)

It also runs the reference's two field kernels that its registration never calls
(estimate_inverse, interpolate_gradient) on seeded fields (field_ops.npz).
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


def field_inputs(dims, seed):
    """psi for estimate_inverse: -(c + 0.3 (x - c) + noise), c the centre of the grid, so
    that -psi o p stays inside the grid and the 48 sweeps do not collapse onto a corner;
    the initial psi_inv is the identity.  For interpolate_gradient: a N(0, 1) field and
    positions identity + N(0, 1.5) noise, some outside the grid, plus a NaN."""
    r = np.random.Generator(np.random.PCG64(seed))
    X, Y, Z = dims
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    idn = np.stack([x, y, z]).astype(np.float64)
    c = np.array([(X - 1) / 2, (Y - 1) / 2, (Z - 1) / 2]).reshape(3, 1, 1, 1)
    psi = -(c + 0.3 * (idn - c) + r.normal(0, 0.5, idn.shape))
    field = r.normal(0, 1, idn.shape)
    pos = idn + r.normal(0, 1.5, idn.shape)
    pos[:, 0, 0, 0] = np.nan
    f32 = lambda a: a.astype(np.float32)  # noqa: E731
    return f32(psi), f32(idn), f32(field), f32(pos)


FIELD_CASES = {"13x11x9": ((13, 11, 9), 201), "30x22x17": ((30, 22, 17), 202)}


def main(out_dir: Path):
    if not ref_runner.available():
        raise SystemExit("reference cubins missing: build them with oracle/ref_build.py where the reference "
                         "sources are present")
    out_dir.mkdir(parents=True, exist_ok=True)
    only_fields = "--fields-only" in sys.argv
    for name, (dims, seed, kw) in ({} if only_fields else CASES).items():
        P = case_params(dims, kw)
        d = case_inputs(dims, seed)
        r = ref_runner.register(P, d["T"], d["labT"], d["S"], d["labS"])
        pv = np.array([P.max_iter, P.reset_iter, P.max_update_norm, P.rho_0, P.tau, P.w_reg, P.alpha, P.p, P.C],
                      np.float64)
        np.savez_compressed(out_dir / f"{name}.npz", dims=np.array(dims), params=pv, T=d["T"], labT=d["labT"],
                            S=d["S"], labS=d["labS"], **{k: v for k, v in r.items() if k != "iterations"},
                            iterations=np.array(r["iterations"]))
        print(f"{name}: {r['iterations']} iterations, last max update norm {r['trace_norm'][-1]:.6g}")
    arrays = {}
    for name, (dims, seed) in FIELD_CASES.items():
        psi, psi_inv0, field, pos = field_inputs(dims, seed)
        arrays[f"{name}_psi"], arrays[f"{name}_psi_inv0"] = psi, psi_inv0
        arrays[f"{name}_field"], arrays[f"{name}_pos"] = field, pos
        arrays[f"{name}_psi_inv48"] = ref_runner.estimate_inverse(psi, psi_inv0, 48)
        arrays[f"{name}_field_o_pos"] = ref_runner.interpolate_gradient(field, pos)
        print(f"field ops {name}: done")
    np.savez_compressed(out_dir / "field_ops.npz", **arrays)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    main(Path(args[0]) if args else ROOT / "tests" / "golden")
