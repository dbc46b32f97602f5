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


# the single-pair workloads: a 64^3 pair (4 label classes, max displacement 3 voxels) and
# the 182x218x182 pair the throughput is quoted on (8 classes, max displacement 6, noise)
PAIR_64CUBE = PairSpec(dims=(64, 64, 64), n_blobs=40, vel_sigma=4.0, max_disp=3.0, n_classes=4, seed=1000)
PAIR_182X218X182 = PairSpec(dims=(182, 218, 182), n_blobs=400, noise=0.01, vel_sigma=6.0, max_disp=6.0, n_classes=8, seed=2000)


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


def make_pair_torch(spec: PairSpec, device="cuda", target=None, source_noise: float = 0.0):
    """The same construction on the GPU with torch (for large cohorts in the benchmark;
    the values differ from make_pair's in rounding).  Returns CUDA tensors T, labT, S,
    labS of shape (Z, Y, X).  With `target` (a (Z, Y, X) tensor) the blobs are skipped and
    that target is warped; `source_noise` adds N(0, source_noise^2) to the source."""
    import torch
    import torch.nn.functional as F

    g = torch.Generator(device="cpu").manual_seed(int(spec.seed))
    X, Y, Z = spec.dims
    dev = torch.device(device)
    zz = torch.arange(Z, device=dev, dtype=torch.float32)[:, None, None]
    yy = torch.arange(Y, device=dev, dtype=torch.float32)[None, :, None]
    xx = torch.arange(X, device=dev, dtype=torch.float32)[None, None, :]
    T = torch.zeros((Z, Y, X), device=dev, dtype=torch.float32)
    lo = torch.tensor([0.0, 0.0, 0.0])
    hi = torch.tensor([X - 1.0, Y - 1.0, Z - 1.0])
    for _ in range(spec.n_blobs if target is None else 0):
        c = lo + (hi - lo) * torch.rand(3, generator=g)
        s = spec.sigma_range[0] + (spec.sigma_range[1] - spec.sigma_range[0]) * float(torch.rand(1, generator=g))
        a = spec.amp_range[0] + (spec.amp_range[1] - spec.amp_range[0]) * float(torch.rand(1, generator=g))
        inv = 1.0 / (2 * s * s)
        T += a * (torch.exp(-(xx - float(c[0])) ** 2 * inv) * torch.exp(-(yy - float(c[1])) ** 2 * inv) *
                  torch.exp(-(zz - float(c[2])) ** 2 * inv))
    T = T.clamp(0.0, 1.0)
    if target is not None:
        T = target.to(dev, torch.float32)
    elif spec.noise > 0:
        T = T + spec.noise * torch.randn((Z, Y, X), generator=g).to(dev)

    def smooth(vol, sigma):
        r = int(3 * sigma + 0.5)
        k = torch.exp(-torch.arange(-r, r + 1, dtype=torch.float32) ** 2 / (2 * sigma * sigma))
        k = (k / k.sum()).to(dev)
        v = vol[None, None]
        v = F.conv3d(F.pad(v, (r, r, 0, 0, 0, 0), mode="replicate"), k.view(1, 1, 1, 1, -1))
        v = F.conv3d(F.pad(v, (0, 0, r, r, 0, 0), mode="replicate"), k.view(1, 1, 1, -1, 1))
        v = F.conv3d(F.pad(v, (0, 0, 0, 0, r, r), mode="replicate"), k.view(1, 1, -1, 1, 1))
        return v[0, 0]

    v = torch.stack([smooth(torch.randn((Z, Y, X), generator=g).to(dev), spec.vel_sigma) for _ in range(3)])
    v *= spec.max_disp / v.pow(2).sum(0).sqrt().max().clamp_min(1e-12)

    def sample(field, disp, mode):
        # field (C, Z, Y, X); disp (3, Z, Y, X) in voxels, components (x, y, z)
        px = (xx + disp[0]) * (2.0 / max(X - 1, 1)) - 1.0
        py = (yy + disp[1]) * (2.0 / max(Y - 1, 1)) - 1.0
        pz = (zz + disp[2]) * (2.0 / max(Z - 1, 1)) - 1.0
        grid = torch.stack([px, py, pz], dim=-1)[None]
        return F.grid_sample(field[None], grid, mode=mode, padding_mode="border", align_corners=True)[0]

    u = v / (2 ** spec.squarings)
    for _ in range(spec.squarings):
        u = u + sample(u, u, "bilinear")
    S = sample(T[None], u, "bilinear")[0]
    if source_noise > 0:
        S = S + source_noise * torch.randn((Z, Y, X), generator=g).to(dev)
    thr = torch.arange(1, spec.n_classes, device=dev, dtype=torch.float32) / spec.n_classes
    labT = torch.bucketize(T.clamp(0.0, 1.0), thr, right=True).to(torch.int16)
    labS = sample(labT[None].float(), u, "nearest")[0].to(torch.int16)
    return dict(T=T.contiguous(), labT=labT.contiguous(), S=S.contiguous(), labS=labS.contiguous())


def cohort_specs(n_pairs: int = 16, seed: int = 3000):
    """The uneven batched cohort: dims drawn per pair (cohort_dims), blobs scaled with
    the volume, maximum displacement uniform in [2, 6] voxels, one seed per pair."""
    rng = np.random.Generator(np.random.PCG64(seed + 1))
    specs = []
    for k, d in enumerate(cohort_dims(n_pairs, seed)):
        n = d[0] * d[1] * d[2]
        specs.append(PairSpec(dims=d, n_blobs=max(40, n // 20000), vel_sigma=4.0,
                              max_disp=float(rng.uniform(2.0, 6.0)), n_classes=4, seed=seed + 100 + k))
    return specs


def shared_target_cohort(n_pairs: int = 32, dims=(160, 192, 160), device="cuda", seed: int = 5000):
    """The shared-target cohort: one target of Gaussian blobs; each source is that target
    warped by its own seeded velocity (Gaussian sigma 5, maximum displacement 5 voxels)
    plus N(0, 0.02) intensity noise; 8 label classes.  Returns a list of dicts as
    make_pair_torch (the target tensors are shared)."""
    n = dims[0] * dims[1] * dims[2]
    base = PairSpec(dims=dims, n_blobs=max(40, n // 18000), vel_sigma=5.0, max_disp=5.0, n_classes=8, seed=seed)
    first = make_pair_torch(base, device)
    out = []
    for k in range(n_pairs):
        sp = PairSpec(**{**base.__dict__, "seed": seed + 1 + k})
        d = make_pair_torch(sp, device, target=first["T"], source_noise=0.02)
        out.append(d)
    return out
