"""The hand-written adjoint kernels on the GPU (fr_sobolev_loss_grad, fr_warp_adjoint)
against the FP64 oracle and central finite differences of the FP64 forward.

The registration is wrapped in a torch.autograd.Function here, in the test harness only:
the library itself is plain CUDA behind the C ABI."""
import ctypes as C

import numpy as np
import pytest

from fastreg_gb300 import Params, _native as N
from oracle import oracle as O
from tests.helpers import images, rng, smooth_noise

pytestmark = pytest.mark.gpu


def _loss_grad(T, S, v0, lam, K, ck, P, want_grad=True):
    import torch
    lib = N.load()
    z, y, x = T.shape
    dims = (C.c_int * 3)(x, y, z)
    loss = C.c_double()
    gl = C.c_double()
    gv = torch.empty_like(v0) if want_grad else None
    rc = lib.fr_sobolev_loss_grad(T.data_ptr(), S.data_ptr(), dims, v0.data_ptr(), float(lam), int(K), int(ck),
                                  P.damping, P.step, P.smooth_sigma, int(P.smooth_width), C.byref(loss),
                                  gv.data_ptr() if want_grad else None, C.byref(gl), None)
    assert rc == N.FR_OK, lib.fr_last_error(None)
    return loss.value, gv, gl.value


def _registration_fn():
    import torch

    class SobolevRegistration(torch.autograd.Function):
        """J(v0, lambda) of a K-iteration sobolev registration; backward runs the
        adjoint kernels."""

        @staticmethod
        def forward(ctx, v0, lam, T, S, K, ck, P):
            J, gv, gl = _loss_grad(T, S, v0.detach().contiguous(), float(lam), K, ck, P)
            ctx.save_for_backward(gv, torch.tensor(gl, dtype=torch.float64))
            return torch.tensor(J, dtype=torch.float64, device=v0.device)

        @staticmethod
        def backward(ctx, gJ):
            gv, gl = ctx.saved_tensors
            return (gJ.to(gv.dtype) * gv, (gJ.cpu() * gl).to(torch.float64), None, None, None, None, None)

    return SobolevRegistration.apply


def test_loss_gradient_against_fp64_oracle_and_finite_differences(cuda):
    import torch
    dims = (24, 20, 18)
    d = images(dims, 21)
    P = Params(volume_dims=dims, solver="sobolev", smooth_sigma=1.5, smooth_width=7, damping=0.9, step=0.5)
    v0 = smooth_noise(rng(2), (3,) + dims[::-1], 0.3)
    lam, K, ck = 0.2, 12, 5
    T, S = (torch.from_numpy(d[k]).to(cuda) for k in ("T", "S"))
    v0_t = torch.from_numpy(v0).to(cuda).requires_grad_(True)
    lam_t = torch.tensor(lam, dtype=torch.float64, requires_grad=True)
    J = _registration_fn()(v0_t, lam_t, T, S, K, ck, P)
    J.backward()
    gv = v0_t.grad.cpu().numpy().astype(np.float64)
    gl = float(lam_t.grad)

    J64, gv64, gl64 = O.sob_loss_grad(P, d["T"], d["S"], v0.astype(np.float64), lam, K)
    J32, _, _ = O.sob_loss_grad(P, d["T"], d["S"], v0, lam, K, False, prec=32)
    J = float(J.detach())
    assert abs(J - J32) <= 1e-9 * abs(J32)          # same FP32 forward, FP64 sums in another order
    assert abs(J - J64) <= 1e-5 * abs(J64)
    assert abs(gl - gl64) <= 1e-4 * abs(gl64), (gl, gl64)
    scale = float(np.abs(gv64).max())
    err = np.abs(gv - gv64).max() / scale
    assert err <= 1e-3, f"dJ/dv0: max |gpu - fp64| / max |grad| = {err:.3g}"

    # central finite differences of the FP64 forward at 64 random voxel components and at
    # lambda.  The model is piecewise smooth (trilinear interpolation has kinks on cell
    # faces); a difference whose step lets any of the ~1e5 sample positions cross a face
    # measures a mix of two slopes, so each check takes the best of three small steps.
    def fd_lambda(eps):
        Jp, _, _ = O.sob_loss_grad(P, d["T"], d["S"], v0.astype(np.float64), lam + eps, K, False)
        Jm, _, _ = O.sob_loss_grad(P, d["T"], d["S"], v0.astype(np.float64), lam - eps, K, False)
        return (Jp - Jm) / (2 * eps)

    errs = [abs(gl - fd_lambda(eps)) / abs(gl) for eps in (1e-6, 1e-7, 1e-8)]
    assert min(errs) <= 1e-4, errs
    r = rng(11)
    bad = []
    for _ in range(64):
        c = int(r.integers(0, 3))
        z, y, x = (int(r.integers(0, n)) for n in v0.shape[1:])
        best = np.inf
        for eps in (1e-6, 1e-7):
            vp = v0.astype(np.float64)
            vm = vp.copy()
            vp[c, z, y, x] += eps
            vm[c, z, y, x] -= eps
            Jp, _, _ = O.sob_loss_grad(P, d["T"], d["S"], vp, lam, K, False)
            Jm, _, _ = O.sob_loss_grad(P, d["T"], d["S"], vm, lam, K, False)
            fdv = (Jp - Jm) / (2 * eps)
            best = min(best, abs(fdv - gv[c, z, y, x]) / max(abs(fdv), 1e-2 * scale))
        if best > 1e-4:
            bad.append((c, z, y, x, best))
    assert not bad, bad[:4]


def test_checkpointing_does_not_change_the_gradient(cuda):
    import torch
    dims = (16, 14, 12)
    d = images(dims, 4)
    P = Params(volume_dims=dims, solver="sobolev", smooth_sigma=1.5, smooth_width=7, damping=0.9, step=0.5)
    v0 = torch.from_numpy(smooth_noise(rng(3), (3,) + dims[::-1], 0.2)).to(cuda)
    T, S = (torch.from_numpy(d[k]).to(cuda) for k in ("T", "S"))
    J1, g1, l1 = _loss_grad(T, S, v0, 0.1, 10, 10, P)
    J2, g2, l2 = _loss_grad(T, S, v0, 0.1, 10, 3, P)
    assert abs(J1 - J2) <= 1e-12 * abs(J1)  # FP64 atomics add the block sums in any order
    assert torch.allclose(g1, g2, rtol=1e-5, atol=1e-6 * float(g1.abs().max()))
    assert abs(l1 - l2) <= 1e-6 * abs(l1)


def test_warp_adjoint(cuda):
    import torch
    lib = N.load()
    dims = (20, 18, 16)
    r = rng(9)
    img = r.normal(0, 1, dims[::-1]).astype(np.float32)
    pos = np.stack(np.meshgrid(np.arange(16), np.arange(18), np.arange(20), indexing="ij")[::-1]).astype(np.float32)
    pos = pos + r.uniform(-2.5, 2.5, pos.shape).astype(np.float32)
    wbar = r.normal(0, 1, dims[::-1]).astype(np.float32)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)  # noqa: E731
    pb, ib = torch.empty((3,) + dims[::-1], device=cuda), torch.empty(dims[::-1], device=cuda)
    cd = (C.c_int * 3)(*dims)
    assert lib.fr_warp_adjoint(t(pos).data_ptr(), t(img).data_ptr(), t(wbar).data_ptr(), cd, pb.data_ptr(),
                               ib.data_ptr(), None) == N.FR_OK
    pb64, ib64 = O.warp_adjoint(pos, img, wbar)
    assert np.abs(pb.cpu().numpy() - pb64).max() <= 1e-5 * max(1.0, np.abs(pb64).max())
    assert np.abs(ib.cpu().numpy() - ib64).max() <= 1e-5 * max(1.0, np.abs(ib64).max())


def test_hypergradient_tuned_cohort(cuda):
    """fastreg_gb300.hypertune: per-pair W_REG from hypergradient steps through short
    unrolled registrations, then one batched registration with those weights -- the same
    bits as each pair registered alone with its weight."""
    import torch
    from fastreg_gb300 import FastReg, Params, _native as N
    from fastreg_gb300.hypertune import register_cohort_tuned, tune_w_reg
    dims_list = [(24, 20, 18), (20, 22, 16)]
    pairs_np = [images(d, 1200 + k) for k, d in enumerate(dims_list)]
    kw = dict(no_labels=4, max_iter=15, solver="sobolev", smooth_sigma=1.5, smooth_width=7, damping=0.9, step=0.5,
              w_reg=0.2)
    P = Params(volume_dims=dims_list[0], **kw)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)  # noqa: E731
    lam, hist = tune_w_reg(t(pairs_np[0]["T"]), t(pairs_np[0]["S"]), P, steps=2, iters=5, checkpoint_every=2)
    assert len(hist) == 2 and all(np.isfinite(h[1]) and np.isfinite(h[2]) for h in hist)
    assert lam > 0 and np.isfinite(lam) and lam != 0.2
    fr = FastReg(P)
    work = [tuple(t(p[k]) for k in ("T", "labT", "S", "labS")) for p in pairs_np]
    weights = register_cohort_tuned(fr, work, P, steps=2, iters=5, checkpoint_every=2)
    for k, (d, p) in enumerate(zip(dims_list, pairs_np)):
        alone = FastReg(Params(volume_dims=d, **{**kw, "w_reg": float(np.float32(weights[k]))}))
        alone(*(t(p[q]) for q in ("T", "labT", "S", "labS")))
        assert torch.equal(fr.get_field(N.FR_FIELD_PSI, pair=k), alone.get_field(N.FR_FIELD_PSI)), k
        alone.close()
    fr.close()


@pytest.mark.slow
def test_adjoint_at_128cube_50_iterations(cuda):
    """The differentiated workload at its stated size: the 128^3 pair (blobs, max
    displacement 4 voxels), 50 unrolled sobolev iterations, checkpoints every 10,
    J = SSD + 0.1 |m_K|^2.

    - Against the FP32 oracle (the same forward arithmetic, so the same trajectory):
      J within 1e-9, dJ/dlambda and dJ/dv0 within 1e-5 relative (the reverse sweeps add
      in different orders).
    - Against the FP64 oracle: J within 1e-5 and dJ/dlambda within 1e-4 relative; dJ/dv0
      no further from it than the FP32 oracle is.  FP32 and FP64 trajectories put a few
      sample positions on different sides of a cell face, where the interpolant's slope
      jumps: about 1000 of the 6.3 M components carry nearly all of that distance
      (6.4e-4 in L2 for either FP32 computation).
    - Against central finite differences of the FP64 forward, every relative error <= 1e-4:
      at lambda, along a random direction over 64 voxels, and at 8 voxel components with
      large gradients.  J is piecewise smooth (a kink wherever a sample crosses a cell
      face); a difference whose step straddles a kink measures a mix of two slopes, so each
      check tries eps = 1e-3 first and then smaller steps, down to where the FP64 forward's
      rounding would show."""
    import json
    import os
    import torch
    from fastreg_gb300 import synthetic as sy
    dims = (128, 128, 128)
    d = sy.make_pair(sy.PairSpec(dims=dims, n_blobs=40, vel_sigma=4.0, max_disp=4.0, n_classes=4, seed=4000))
    P = Params(volume_dims=dims, solver="sobolev", smooth_sigma=1.5, smooth_width=7, damping=0.9, step=0.5)
    v0 = (0.05 * rng(4001).normal(0.0, 1.0, (3,) + dims[::-1])).astype(np.float32)
    lam, K, ck = 0.2, 50, 10
    T, S = (torch.from_numpy(d[k]).to(cuda) for k in ("T", "S"))
    J, gv_t, gl = _loss_grad(T, S, torch.from_numpy(v0).to(cuda), lam, K, ck, P)
    gv = gv_t.cpu().numpy().astype(np.float64)
    v64 = v0.astype(np.float64)
    J64, gv64, gl64 = O.sob_loss_grad(P, d["T"], d["S"], v64, lam, K)
    J32, gv32, gl32 = O.sob_loss_grad(P, d["T"], d["S"], v0, lam, K, True, prec=32)
    gv32 = gv32.astype(np.float64)

    def fwd(v, l):
        return O.sob_loss_grad(P, d["T"], d["S"], v, l, K, False)[0]

    def fd(f, target, steps):
        """central differences of f at each step until one is within 1e-4 of target"""
        tried = {}
        for eps in steps:
            g = (f(eps) - f(-eps)) / (2 * eps)
            tried[eps] = abs(target - g) / abs(g)
            if tried[eps] <= 1e-4:
                break
        return tried

    l2 = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    rec = {"J_rel_fp32": abs(J - J32) / abs(J32), "dlambda_rel_fp32": abs(gl - gl32) / abs(gl32),
           "dv0_rel_l2_fp32": l2(gv, gv32),
           "J_rel_fp64": abs(J - J64) / abs(J64), "dlambda_rel_fp64": abs(gl - gl64) / abs(gl64),
           "dv0_rel_l2_fp64": l2(gv, gv64), "dv0_rel_l2_fp32_oracle_vs_fp64": l2(gv32, gv64)}
    rec["fd_lambda"] = fd(lambda e: fwd(v64, lam + e), gl, (1e-3, 1e-5, 1e-7, 1e-8, 1e-9, 1e-10))
    r = rng(4002)
    direction = np.zeros_like(v64)
    flat = r.choice(v64[0].size, 64, replace=False)
    for c in range(3):
        direction[c].flat[flat] = r.choice([-1.0, 1.0], 64)
    rec["fd_direction_64_voxels"] = fd(lambda e: fwd(v64 + e * direction, lam), float((gv * direction).sum()),
                                       (1e-3, 1e-5, 1e-7, 1e-8))
    big = np.flatnonzero(np.abs(gv64) >= 0.1 * np.abs(gv64).max())
    rec["fd_voxels"] = {}
    for idx in r.choice(big, 8, replace=False):
        e_i = np.zeros(v64.size)
        e_i[idx] = 1.0
        e_i = e_i.reshape(v64.shape)
        rec["fd_voxels"][int(idx)] = fd(lambda e: fwd(v64 + e * e_i, lam), float(gv.flat[idx]), (1e-3, 1e-5, 1e-7))
    print(json.dumps(rec))
    out = os.environ.get("FASTREG_RECORD_DIR")
    if out:
        with open(os.path.join(out, "adjoint_128cube.json"), "w") as f:
            json.dump(rec, f, indent=1)
    assert rec["J_rel_fp32"] <= 1e-9
    assert rec["dlambda_rel_fp32"] <= 1e-5
    assert rec["dv0_rel_l2_fp32"] <= 1e-5
    assert rec["J_rel_fp64"] <= 1e-5
    assert rec["dlambda_rel_fp64"] <= 1e-4
    assert rec["dv0_rel_l2_fp64"] <= 1.02 * rec["dv0_rel_l2_fp32_oracle_vs_fp64"] + 1e-6
    assert min(rec["fd_lambda"].values()) <= 1e-4, rec["fd_lambda"]
    assert min(rec["fd_direction_64_voxels"].values()) <= 1e-4, rec["fd_direction_64_voxels"]
    for k, v in rec["fd_voxels"].items():
        assert min(v.values()) <= 1e-4, (k, v)
