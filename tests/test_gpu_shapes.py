"""Volumes of extreme shape on the GPU against the oracle: thin along one axis and long
along another, down to the smallest accepted size (4 voxels per axis, a 2-voxel
interior), registered as one cohort with either staging and compared pair by pair with
the oracle bit for bit.  An empty cohort and a volume below the minimum are refused with
a status, and the handle registers correctly afterwards."""
import numpy as np
import pytest

from fastreg_gb300 import FastReg, Params, _native as N
from oracle import oracle as O
from tests.helpers import assert_bitexact, images

pytestmark = pytest.mark.gpu

# (X, Y, Z): one voxel-pitch chunk wide in x (4), rows of one or two tiles, 70 slices, a
# row pitch padded from 97 to 100, and the minimum cube
SHAPES = [(4, 45, 5), (70, 4, 6), (5, 6, 70), (97, 5, 4), (4, 4, 4)]


def _to(dev, a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _check_pair(solver, P, p, buf, psi, what):
    if solver == "reference":
        o = O.ref_register(P, p["T"], p["labT"], p["S"], p["labS"])
        assert_bitexact(psi, o["psi"], f"{what} psi")
        assert_bitexact(buf[0].cpu().numpy(), o["out_T"], f"{what} T o psi_inv")
        assert_bitexact(buf[1].cpu().numpy(), o["out_labT"], f"{what} labels T o psi_inv")
        assert_bitexact(buf[2].cpu().numpy(), o["out_S"], f"{what} S o psi")
        assert_bitexact(buf[3].cpu().numpy(), o["out_labS"], f"{what} labels S o psi")
    else:
        o = O.sob_register(P, p["T"], p["S"])
        assert_bitexact(psi, o["phi"], f"{what} phi")
        assert_bitexact(buf[2].cpu().numpy(), O.warp(o["phi"], p["S"]), f"{what} S o phi")
        assert_bitexact(buf[3].cpu().numpy(), O.warp_nearest_label(o["phi"], p["labS"]), f"{what} labels")


@pytest.mark.parametrize("staging", [1, 2])
@pytest.mark.parametrize("solver", ["reference", "sobolev"])
def test_extreme_shapes_as_one_cohort(cuda, solver, staging):
    kw = dict(no_labels=4, max_iter=15, alpha=0.02, solver=solver, step=0.5, damping=0.9, staging=staging)
    pairs_np = [images(d, 1700 + k) for k, d in enumerate(SHAPES)]
    fr = FastReg(Params(volume_dims=SHAPES[0], **kw))
    bufs = [tuple(_to(cuda, p[k]) for k in ("T", "labT", "S", "labS")) for p in pairs_np]
    fr.register_batch(bufs)
    for k, (d, p) in enumerate(zip(SHAPES, pairs_np)):
        psi = fr.get_field(N.FR_FIELD_PSI, pair=k).cpu().numpy()
        _check_pair(solver, Params(volume_dims=d, **kw), p, bufs[k], psi, f"pair {k} {d}")
        assert fr.stats(pair=k).iterations == 15
    fr.close()


def test_empty_and_undersized_cohorts_are_refused(cuda):
    from fastreg_gb300._native import FastRegError
    kw = dict(no_labels=4, max_iter=10, alpha=0.02)
    fr = FastReg(Params(volume_dims=(12, 10, 9), **kw))
    with pytest.raises(FastRegError, match="at least one pair"):
        fr.register_batch([])
    small = images((3, 10, 10), 1800)
    with pytest.raises(FastRegError, match="< 4"):
        fr.register_batch([tuple(_to(cuda, small[k]) for k in ("T", "labT", "S", "labS"))])
    # the handle still works
    p = images((12, 10, 9), 1801)
    buf = tuple(_to(cuda, p[k]) for k in ("T", "labT", "S", "labS"))
    fr(*buf)
    _check_pair("reference", Params(volume_dims=(12, 10, 9), **kw), p, buf,
                fr.get_field(N.FR_FIELD_PSI).cpu().numpy(), "after the refusals")
    fr.close()
