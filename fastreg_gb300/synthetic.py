"""Seeded synthetic registration pairs (stand-ins for the MRI pairs of the paper).

A target T is a clipped sum of Gaussian blobs; a smooth stationary velocity
(i.i.d. N(0,1) per component, Gaussian-smoothed, scaled to a maximum
displacement) is exponentiated by scaling and squaring; the source is
S = T o (x + u) (trilinear) and its labels are T's threshold classes warped
nearest-neighbour with the same map.  FP64 generation (PCG64), FP32 output.
Arrays are (Z, Y, X), x fastest.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
from scipy import ndimage


@dataclass
class PairSpec:
    dims: tuple            # (X, Y, Z)
    n_blobs: int = 40
    sigma_range: tuple = (3.0, 8.0)
    amp_range: tuple = (0.2, 1.0)
    noise: float = 0.0     # std of additive N(0, noise^2) intensity noise on the target
    vel_sigma: float = 4.0
    max_disp: float = 3.0
    n_classes: int = 4
    squarings: int = 6
    seed: int = 1000


# the workloads of the benchmark configurations
CFG1 = PairSpec(dims=(64, 64, 64), n_blobs=40, vel_sigma=4.0, max_disp=3.0, n_classes=4, seed=1000)
CFG2 = PairSpec(dims=(182, 218, 182), n_blobs=400, noise=0.01, vel_sigma=6.0, max_disp=6.0, n_classes=8, seed=2000)


def blobs(dims, n, sigma_range, amp_range, rng) -> np.ndarray:
    X, Y, Z = dims
    vol = np.zeros((Z, Y, X), np.float64)
    for _ in range(n):
        c = rng.uniform([0, 0, 0], [X - 1, Y - 1, Z - 1])
        s = rng.uniform(*sigma_range)
        a = rng.uniform(*amp_range)
        r = int(np.ceil(3.5 * s))
        lo = np.maximum(np.floor(c).astype(int) - r, 0)
        hi = np.minimum(np.floor(c).astype(int) + r + 1, [X, Y, Z])
        xs = np.arange(lo[0], hi[0]) - c[0]
        ys = np.arange(lo[1], hi[1]) - c[1]
        zs = np.arange(lo[2], hi[2]) - c[2]
        gx = np.exp(-xs ** 2 / (2 * s * s))
        gy = np.exp(-ys ** 2 / (2 * s * s))
        gz = np.exp(-zs ** 2 / (2 * s * s))
        vol[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] += a * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return vol


def _sample(field: np.ndarray, coords: np.ndarray, order: int) -> np.ndarray:
    return ndimage.map_coordinates(field, coords, order=order, mode="nearest")


def exp_velocity(v: np.ndarray, squarings: int) -> np.ndarray:
    """Displacement of exp(v) by scaling and squaring; v is (3, Z, Y, X) in voxels
    (component order x, y, z)."""
    Z, Y, X = v.shape[1:]
    grid = np.stack(np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")).astype(np.float64)
    u = v / (2 ** squarings)
    for _ in range(squarings):
        coords = grid + np.stack([u[2], u[1], u[0]])  # (z, y, x) sample positions
        u = u + np.stack([_sample(u[c], coords, 1) for c in range(3)])
    return u


def make_pair(spec: PairSpec):
    """Returns dict(T, labT, S, labS, u) with T/S float32, labels int16, u the true
    displacement (3, Z, Y, X) float32 (x, y, z components)."""
    rng = np.random.Generator(np.random.PCG64(spec.seed))
    X, Y, Z = spec.dims
    T = blobs(spec.dims, spec.n_blobs, spec.sigma_range, spec.amp_range, rng)
    T = np.clip(T, 0.0, 1.0)
    if spec.noise > 0:
        T = T + rng.normal(0.0, spec.noise, T.shape)
    v = rng.normal(0.0, 1.0, (3, Z, Y, X))
    for c in range(3):
        v[c] = ndimage.gaussian_filter(v[c], spec.vel_sigma, mode="nearest")
    mag = np.sqrt((v ** 2).sum(0)).max()
    v *= spec.max_disp / max(mag, 1e-12)
    u = exp_velocity(v, spec.squarings)
    grid = np.stack(np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")).astype(np.float64)
    coords = grid + np.stack([u[2], u[1], u[0]])
    S = _sample(T, coords, 1)
    thr = np.arange(1, spec.n_classes) / spec.n_classes
    labT = np.digitize(np.clip(T, 0.0, 1.0), thr).astype(np.int16)
    labS = _sample(labT.astype(np.float64), coords, 0).astype(np.int16)
    return dict(T=T.astype(np.float32), labT=labT, S=S.astype(np.float32), labS=labS, u=u.astype(np.float32))


def cohort_dims(n_pairs: int, seed: int = 3000):
    """Dims of the uneven batched cohort: X in {96,128,160,192}, Y in {112,160,224},
    Z in {96,128,192}, drawn per pair."""
    rng = np.random.Generator(np.random.PCG64(seed))
    xs, ys, zs = (96, 128, 160, 192), (112, 160, 224), (96, 128, 192)
    return [(int(rng.choice(xs)), int(rng.choice(ys)), int(rng.choice(zs))) for _ in range(n_pairs)]
