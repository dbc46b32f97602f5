"""Shared helpers of the parity tests: seeded states and comparisons."""
from __future__ import annotations

import numpy as np


def rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def identity(dims):
    X, Y, Z = dims
    z, y, x = np.meshgrid(np.arange(Z), np.arange(Y), np.arange(X), indexing="ij")
    return np.stack([x, y, z]).astype(np.float32)


def smooth_noise(r, shape, scale, sigma=2.0):
    from scipy import ndimage
    a = r.normal(0.0, 1.0, shape)
    if a.ndim == 4:
        for c in range(a.shape[0]):
            a[c] = ndimage.gaussian_filter(a[c], sigma, mode="nearest")
    else:
        a = ndimage.gaussian_filter(a, sigma, mode="nearest")
    m = np.abs(a).max()
    return (a * (scale / max(m, 1e-12))).astype(np.float32)


def random_state(dims, seed, disp=1.5, vel=0.05):
    """A plausible mid-registration state: psi/psi_inv = identity + smooth
    displacement, v smooth, rho around 1; boundary kept as the solver keeps it
    (identity psi/psi_inv, v = 0, rho = rho_0 on the 1-voxel shell)."""
    r = rng(seed)
    X, Y, Z = dims
    idn = identity(dims)
    psi = idn + smooth_noise(r, (3, Z, Y, X), disp)
    pinv = idn + smooth_noise(r, (3, Z, Y, X), disp)
    v = smooth_noise(r, (3, Z, Y, X), vel)
    rho = (1.0 + smooth_noise(r, (Z, Y, X), 0.1)).astype(np.float32)
    shell = np.ones((Z, Y, X), bool)
    shell[1:-1, 1:-1, 1:-1] = False
    for c in range(3):
        psi[c][shell] = idn[c][shell]
        pinv[c][shell] = idn[c][shell]
        v[c][shell] = 0.0
    rho[shell] = 1.0
    return dict(psi=psi, psi_inv=pinv, v=v, rho=rho)


def images(dims, seed, n_classes=4):
    from fastreg_gb300 import synthetic as sy
    X, Y, Z = dims
    spec = sy.PairSpec(dims=dims, n_blobs=max(4, X * Y * Z // 6000), vel_sigma=2.0,
                       max_disp=min(3.0, min(dims) / 6), n_classes=n_classes, seed=seed)
    return sy.make_pair(spec)


def assert_bitexact(a, b, what=""):
    a = np.asarray(a)
    b = np.asarray(b)
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    if a.dtype.kind == "f":
        same = (a.view(np.uint32 if a.dtype == np.float32 else np.uint64) ==
                b.astype(a.dtype).view(np.uint32 if a.dtype == np.float32 else np.uint64))
        # +0 and -0 compare equal as values; bit patterns are what we check, NaN too
        bad = ~same
    else:
        bad = a != b
    n = int(bad.sum())
    if n:
        idx = np.argwhere(bad)[:5]
        ex = [(tuple(i), a[tuple(i)], b[tuple(i)]) for i in idx]
        raise AssertionError(f"{what}: {n} of {a.size} elements differ, e.g. {ex}")


def rel_err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), 1e-30)
