"""Known-answer tests of the CPU oracle (runs without a GPU)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import assert_bitexact, identity, images, random_state, rel_err


def test_identity_warp_is_exact_copy():
    r = np.random.Generator(np.random.PCG64(1))
    dims = (9, 7, 5)
    img = r.normal(0, 1, (5, 7, 9)).astype(np.float32)
    lab = r.integers(0, 5, (5, 7, 9)).astype(np.int16)
    out, out_lab = O.warp(identity(dims), img, lab)
    assert np.array_equal(out, img)
    assert np.array_equal(out_lab, lab)


def test_translation_warp_linear_image_is_exact():
    """trilinear interpolation reproduces a linear image exactly (interior shift)."""
    dims = (16, 12, 10)
    pos = identity(dims)
    z, y, x = np.meshgrid(np.arange(10), np.arange(12), np.arange(16), indexing="ij")
    img = (0.5 * x + 0.25 * y - 0.125 * z).astype(np.float32)
    shift = np.array([0.5, 0.25, 0.75], np.float32)[:, None, None, None]
    p = pos + shift
    out = O.warp(p, img)
    inner = (slice(0, 9), slice(0, 11), slice(0, 15))
    expect = 0.5 * (x + 0.5) + 0.25 * (y + 0.25) - 0.125 * (z + 0.75)
    assert np.abs(out[inner] - expect[inner]).max() < 1e-5


def test_floor_corner_label():
    """labels come from the floor corner of the clamped position, not the nearest voxel
    (include/cuda/cuda_utils.hpp:81)."""
    dims = (4, 4, 4)
    lab = np.arange(64, dtype=np.int16).reshape(4, 4, 4)
    img = np.zeros((4, 4, 4), np.float32)
    pos = identity(dims) + np.float32(0.9)
    _, out_lab = O.warp(pos, img, lab)
    assert out_lab[0, 0, 0] == lab[0, 0, 0]      # 0.9 -> floor 0, not round 1
    pos = identity(dims) - np.float32(5)         # clamped to 0
    _, out_lab = O.warp(pos, img, lab)
    assert (out_lab == lab[0, 0, 0]).all()


def test_laplacian_of_identity_is_zero_and_boundary_zero():
    dims = (8, 7, 6)
    L = O.ref_laplacian(identity(dims))
    assert (L == 0).all()
    psi = identity(dims) + np.float32(0.0)
    psi[0, 3, 3, 3] += 1.0
    L = O.ref_laplacian(psi)
    assert L[0, 3, 3, 3] == 6.0 and L[0, 3, 3, 4] == -1.0


def test_reference_det_is_the_misparenthesised_one():
    """det(J) of include/cuda/cuda_utils.hpp:389-396 as written: 1 at identity, and
    (m00 m11 m22 + m10 m21 m02 + m20 m01 m12) - ((m02 m11 + m20)(m12 m21 m00) + m22 m01 m10)."""
    dims = (5, 5, 5)
    pinv = identity(dims)
    assert O.ref_det_field(pinv)[2, 2, 2] == 1.0
    # a linear map psi_inv = A x gives J = A everywhere in the interior
    A = np.array([[1.1, 0.2, 0.3], [0.4, 0.9, 0.1], [0.2, 0.5, 1.3]])
    idn = identity(dims).astype(np.float64)
    lin = np.einsum("rc,czyx->rzyx", A, idn).astype(np.float32)
    got = O.ref_det_field(lin, prec=64)[2, 2, 2]
    m = A
    want = (m[0, 0] * m[1, 1] * m[2, 2] + m[1, 0] * m[2, 1] * m[0, 2] + m[2, 0] * m[0, 1] * m[1, 2]) - \
           ((m[0, 2] * m[1, 1] + m[2, 0]) * (m[1, 2] * m[2, 1] * m[0, 0]) + m[2, 2] * m[0, 1] * m[1, 0])
    assert abs(got - want) < 1e-6
    assert abs(got - np.linalg.det(A)) > 1e-2  # it is not the true determinant


def test_fold_count_of_a_folded_map():
    """a map that reverses x over a slab folds exactly there: det(I + J_u) <= 0."""
    dims = (12, 6, 6)
    psi = identity(dims)
    psi[0, :, :, 4:8] = psi[0, :, :, 4:8][..., ::-1].copy()  # x reversed on columns 4..7
    J, det = O.deformation_jacobian(psi)
    folded = det <= 0
    assert folded[:, :, 4:8].any()
    assert not folded[:, :, :3].any() and not folded[:, :, 9:].any()
    st = O.stats(np.zeros((6, 6, 12), np.float32), np.zeros((6, 6, 12), np.int16), np.zeros((6, 6, 12), np.float32),
                 np.zeros((6, 6, 12), np.int16), psi, 2)
    assert st["folds"] == int(folded.sum())


def test_identity_state_is_a_fixed_point_without_forcing():
    """T == S and v = 0: the flow stays at the identity."""
    dims = (10, 9, 8)
    d = images(dims, 3)
    from fastreg_gb300 import Params
    P = Params(volume_dims=dims, no_labels=4, max_iter=10, alpha=0.05, w_reg=0.2)
    o = O.ref_register(P, d["T"], d["labT"], d["T"], d["labT"])
    assert np.abs(o["psi"] - identity(dims)).max() == 0
    assert np.array_equal(o["out_S"], d["T"])
    assert np.array_equal(o["out_labS"], d["labT"])


def test_fp32_oracle_tracks_fp64_oracle():
    dims = (20, 18, 16)
    d = images(dims, 8)
    from fastreg_gb300 import Params
    P = Params(volume_dims=dims, no_labels=4, max_iter=40, alpha=0.02)
    o32 = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"])
    o64 = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"], prec=64)
    assert rel_err(o32["psi"], o64["psi"]).max() < 1e-5
    assert rel_err(o32["psi_inv"], o64["psi_inv"]).max() < 1e-5
    # floor-corner labels flip only where psi sits within rounding of an integer
    # (psi starts at the identity, so most positions are near integers)
    diff = o32["out_labS"] != o64["out_labS"]
    frac = np.abs(o64["psi"] - np.round(o64["psi"])).min(axis=0)
    assert (frac[diff] < 1e-4).all()


def test_one_step_boundary_untouched():
    dims = (11, 9, 8)
    d = images(dims, 5)
    st = random_state(dims, 6)
    k = O.ref_coef(0.05, 0.1, 2.0, 0.25, 0.2, 0.2)
    L = O.ref_laplacian(st["psi"])
    rho_n, v_n, pinv_n = O.ref_pass_a(k, d["S"], d["T"], False, st["rho"], st["v"], st["psi_inv"], L)
    shell = np.ones(dims[::-1], bool)
    shell[1:-1, 1:-1, 1:-1] = False
    assert np.array_equal(rho_n[shell], st["rho"][shell])
    for c in range(3):
        assert np.array_equal(v_n[c][shell], st["v"][c][shell])
        assert np.array_equal(pinv_n[c][shell], st["psi_inv"][c][shell])
    assert not np.array_equal(v_n, st["v"])


def test_sobolev_gradient_matches_finite_differences():
    """the sobolev data gradient is the derivative of 0.5 sum (S(phi) - T)^2 (FP64)."""
    dims = (10, 9, 8)
    d = images(dims, 12)
    phi = identity(dims).astype(np.float64) + 0.3
    g, e, _ = O.sob_grad(d["S"], d["T"], phi, prec=64)
    r = np.random.Generator(np.random.PCG64(0))
    for _ in range(10):
        c = int(r.integers(0, 3))
        z, y, x = (int(r.integers(1, n - 2)) for n in dims[::-1])
        eps = 1e-4
        p1 = phi.copy(); p1[c, z, y, x] += eps
        p2 = phi.copy(); p2[c, z, y, x] -= eps
        _, e1, _ = O.sob_grad(d["S"], d["T"], p1, prec=64)
        _, e2, _ = O.sob_grad(d["S"], d["T"], p2, prec=64)
        fd = (e1 - e2) / (2 * eps)
        assert abs(fd - g[c, z, y, x]) <= 1e-6 + 1e-4 * abs(fd)


def test_gaussian_taps():
    t = O.gaussian_taps(1.5, 7)
    assert abs(float(t.sum()) - 1.0) < 1e-6
    assert np.allclose(t, t[::-1])
    assert t[3] == t.max()
