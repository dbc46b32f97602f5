"""The FP64 oracle of the differentiated sobolev registration against central finite
differences (runs without a GPU).

The model is piecewise smooth: trilinear interpolation has kinks on the cell faces and
the starting positions (the identity) sit exactly on them.  A finite difference with a
step that lets a sample cross a face measures the average of two one-sided slopes, so
the comparison uses a step of 1e-6 in FP64 (with 1e-3, about a quarter of random
voxels straddle a kink)."""
import numpy as np

from fastreg_gb300 import Params
from oracle import oracle as O
from tests.helpers import images, rng, smooth_noise


def _case(dims=(16, 14, 12), K=10):
    d = images(dims, 5)
    P = Params(volume_dims=dims, solver="sobolev", smooth_sigma=1.5, smooth_width=7, damping=0.9, step=0.5)
    v0 = smooth_noise(rng(1), (3,) + dims[::-1], 0.3).astype(np.float64)
    return d, P, v0, 0.2, K


def test_adjoint_matches_finite_differences():
    d, P, v0, lam, K = _case()
    J, gv, gl = O.sob_loss_grad(P, d["T"], d["S"], v0, lam, K)
    eps = 1e-6
    Jp, _, _ = O.sob_loss_grad(P, d["T"], d["S"], v0, lam + eps, K, False)
    Jm, _, _ = O.sob_loss_grad(P, d["T"], d["S"], v0, lam - eps, K, False)
    fd = (Jp - Jm) / (2 * eps)
    assert abs(fd - gl) <= 1e-4 * abs(fd), (fd, gl)
    r = rng(7)
    scale = float(np.abs(gv).max())
    for _ in range(32):
        c = int(r.integers(0, 3))
        z, y, x = (int(r.integers(0, n)) for n in v0.shape[1:])
        vp = v0.copy()
        vp[c, z, y, x] += eps
        vm = v0.copy()
        vm[c, z, y, x] -= eps
        Jp, _, _ = O.sob_loss_grad(P, d["T"], d["S"], vp, lam, K, False)
        Jm, _, _ = O.sob_loss_grad(P, d["T"], d["S"], vm, lam, K, False)
        fd = (Jp - Jm) / (2 * eps)
        assert abs(fd - gv[c, z, y, x]) <= 1e-4 * max(abs(fd), 1e-3 * scale), (c, z, y, x, fd, gv[c, z, y, x])


def test_loss_is_the_registration_energy():
    """J's data term is the SSD of the sobolev registration run with momentum m_0 = v0."""
    d, P, v0, lam, K = _case()
    J, _, _ = O.sob_loss_grad(P, d["T"], d["S"], np.zeros_like(v0), lam, K, False)
    P2 = Params(**{**P.__dict__, "max_iter": K, "w_reg": lam, "max_update_norm": -1.0})
    o = O.sob_register(P2, d["T"], d["S"], prec=64)
    W = O.warp_sob(o["phi"], d["S"])
    e = 0.5 * float(((W - d["T"].astype(np.float64)) ** 2).sum()) + 0.1 * float((o["m"] ** 2).sum())
    assert abs(J - e) <= 1e-12 * abs(e)


def test_warp_adjoint_matches_finite_differences():
    dims = (10, 9, 8)
    r = rng(3)
    img = r.normal(0, 1, dims[::-1])
    pos = np.stack(np.meshgrid(np.arange(8), np.arange(9), np.arange(10), indexing="ij")[::-1]).astype(np.float64)
    pos = pos + r.uniform(-0.45, 0.45, pos.shape)
    wbar = r.normal(0, 1, dims[::-1])
    pb, ib = O.warp_adjoint(pos, img, wbar)
    f = lambda p, im: float((O.warp_sob(p, im) * wbar).sum())  # noqa: E731
    eps = 1e-6
    for _ in range(16):
        c = int(r.integers(0, 3))
        z, y, x = (int(r.integers(1, n - 1)) for n in dims[::-1])
        p1 = pos.copy(); p1[c, z, y, x] += eps
        p2 = pos.copy(); p2[c, z, y, x] -= eps
        fd = (f(p1, img) - f(p2, img)) / (2 * eps)
        assert abs(fd - pb[c, z, y, x]) <= 1e-6 * max(1.0, abs(fd))
        i1 = img.copy(); i1[z, y, x] += 1.0
        assert abs((f(pos, i1) - f(pos, img)) - ib[z, y, x]) <= 1e-9 * max(1.0, abs(ib[z, y, x]))
