"""Fold counts on the GPU where folds exist: a map loaded into a handle with
fr_set_field(FR_FIELD_PSI), then fr_finish (finalize_kernel), against the oracle's
statistics of the same map -- the fold count (#voxels with det(I + J_u) <= 0, the
correct determinant) exact and nonzero, the energies within 1e-12 relative, the warped
images and labels bit-exact."""
import numpy as np
import pytest

from fastreg_gb300 import FastReg, Params, _native as N
from oracle import oracle as O
from tests.helpers import assert_bitexact, identity, images, rel_err, rng, smooth_noise

pytestmark = pytest.mark.gpu


def _to(dev, a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def slab_reversal(dims):
    """x reversed on columns 4..7 of every row: folds exactly on that slab (the
    oracle's known-answer case)."""
    psi = identity(dims)
    psi[0, :, :, 4:8] = psi[0, :, :, 4:8][..., ::-1].copy()
    return psi


def random_folded(dims, seed, disp):
    """identity + a rough random displacement large enough to fold in places"""
    psi = identity(dims) + smooth_noise(rng(seed), (3,) + dims[::-1], disp, sigma=1.0)
    return psi.astype(np.float32)


CASES = [((12, 6, 6), "slab", 0), ((40, 36, 30), "random", 3), ((33, 17, 20), "random", 4),
         ((64, 48, 40), "random", 5)]


@pytest.mark.parametrize("dims,kind,seed", CASES)
def test_fold_count_with_folds_present(cuda, dims, kind, seed):
    d = images(dims, 50 + seed)
    psi = slab_reversal(dims) if kind == "slab" else random_folded(dims, seed, disp=4.0)
    P = Params(volume_dims=dims, no_labels=4, max_iter=4, alpha=0.05)
    fr = FastReg(P)
    iT, lT, iS, lS = (_to(cuda, d[k]) for k in ("T", "labT", "S", "labS"))
    fr.begin([(iT, lT, iS, lS)])
    fr.set_field(N.FR_FIELD_PSI, _to(cuda, psi))
    fr.finish()
    st = fr.stats()

    out_S, out_labS = O.warp(psi, d["S"], d["labS"])
    assert_bitexact(iS.cpu().numpy(), out_S, "S o psi")
    assert_bitexact(lS.cpu().numpy(), out_labS, "labels S o psi")
    # no iteration ran: the target is left as it is (T o psi_inv is written by the
    # iterations, src/fastreg/cuda/solver.cu:402)
    assert_bitexact(iT.cpu().numpy(), d["T"], "T")
    assert_bitexact(lT.cpu().numpy(), d["labT"], "labels T")
    os_ = O.stats(d["T"], d["labT"], out_S, out_labS, psi, P.no_labels)
    _, det = O.deformation_jacobian(psi)
    want = int((det <= 0).sum())
    assert want > 0 and os_["folds"] == want  # the map does fold
    assert st.folds == want, f"GPU folds {st.folds} vs oracle {want}"
    assert rel_err(st.e_data, os_["e_data"]) < 1e-12
    assert rel_err(st.e_reg, os_["e_reg"]) < 1e-12
    assert st.dice_inter == list(os_["dice_inter"][:P.no_labels])
    assert st.dice_count == list(os_["dice_count"][:P.no_labels])
    fr.close()
