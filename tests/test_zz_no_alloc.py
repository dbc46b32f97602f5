"""fr_stats_noalloc: the registration statistics for callers that cannot allocate
device memory (for example a process whose GPU memory is owned by another
framework's pool, or a pipeline that forbids cudaMalloc after start-up).

It must give what fr_get_stats gives after fr_register -- SSD and regulariser
energies within 1e-12 relative (the two reductions add the same per-voxel FP64
terms in different orders), fold count and Dice counts exactly -- on two calls in
a row, since every call reuses the library's one scratch array.  This file is
collected last so that a run stopping at its first failure has run every other
test first.

The first call on a device is its set-up (it looks the scratch array up, which under
CUDA's lazy module loading loads it); the device's free memory must not change over
the calls after it.  A folded map checks the fold count where it is not zero."""
import ctypes as C

import numpy as np
import pytest

from fastreg_gb300 import FastReg, Params, _native as N
from oracle import oracle as O
from tests.helpers import identity, images, rel_err, rng, smooth_noise

pytestmark = pytest.mark.gpu


def test_stats_noalloc_matches_fr_get_stats(cuda):
    import torch
    lib = N.load()
    dims = (40, 36, 30)
    d = images(dims, 77)
    P = Params(volume_dims=dims, no_labels=4, max_iter=40, alpha=0.05)
    fr = FastReg(P)
    T0 = torch.from_numpy(d["T"]).to(cuda)
    labT0 = torch.from_numpy(d["labT"]).to(cuda)
    bufs = [T0.clone(), labT0.clone(), torch.from_numpy(d["S"]).to(cuda), torch.from_numpy(d["labS"]).to(cuda)]
    fr(*bufs)
    ref = fr.stats()
    psi = fr.get_field(N.FR_FIELD_PSI)
    warped_S, warped_labS = bufs[2], bufs[3]
    c_dims = (C.c_int * 3)(*dims)
    free_after = []
    for call in range(2):
        out = N.fr_stats()
        rc = lib.fr_stats_noalloc(T0.data_ptr(), labT0.data_ptr(), warped_S.data_ptr(), warped_labS.data_ptr(),
                                  psi.data_ptr(), c_dims, P.no_labels, P.w_reg, C.byref(out), None)
        assert rc == N.FR_OK, lib.fr_last_error(None)
        assert rel_err(out.e_data, ref.e_data) <= 1e-12, call
        assert rel_err(out.e_reg, ref.e_reg) <= 1e-12, call
        assert rel_err(out.energy, ref.energy) <= 1e-12, call
        assert out.folds == ref.folds, call
        assert list(out.dice_inter[:P.no_labels]) == ref.dice_inter, call
        assert list(out.dice_count[:P.no_labels]) == ref.dice_count, call
        assert out.dice_out_of_range == ref.dice_out_of_range, call
        assert out.dice_all == pytest.approx(ref.dice_all, rel=1e-12, nan_ok=True), call
        torch.cuda.synchronize()
        free_after.append(torch.cuda.mem_get_info()[0])
    # the second call allocated nothing on the device
    assert free_after[1] == free_after[0], free_after
    # inputs beyond the limits are refused with a message, before any GPU work
    bad = (C.c_int * 3)(1, 36, 30)
    out = N.fr_stats()
    rc = lib.fr_stats_noalloc(T0.data_ptr(), labT0.data_ptr(), warped_S.data_ptr(), warped_labS.data_ptr(),
                              psi.data_ptr(), bad, P.no_labels, P.w_reg, C.byref(out), None)
    assert rc == N.FR_ERR_INVALID_ARG and b"dimension" in lib.fr_last_error(None)
    rc = lib.fr_stats_noalloc(T0.data_ptr(), labT0.data_ptr(), warped_S.data_ptr(), warped_labS.data_ptr(),
                              psi.data_ptr(), c_dims, 300, P.w_reg, C.byref(out), None)
    assert rc == N.FR_ERR_INVALID_ARG and b"no_labels" in lib.fr_last_error(None)
    fr.close()


def test_stats_noalloc_counts_folds(cuda):
    """A map that folds in places: fr_stats_noalloc's fold count equals the oracle's
    (nonzero), twice in a row."""
    import torch
    lib = N.load()
    dims = (40, 36, 30)
    d = images(dims, 91)
    psi = (identity(dims) + smooth_noise(rng(9), (3,) + dims[::-1], 4.0, sigma=1.0)).astype(np.float32)
    wS, wlabS = O.warp(psi, d["S"], d["labS"])
    os_ = O.stats(d["T"], d["labT"], wS, wlabS, psi, 4)
    assert os_["folds"] > 0
    t = [torch.from_numpy(np.ascontiguousarray(a)).to(cuda) for a in (d["T"], d["labT"], wS, wlabS, psi)]
    c_dims = (C.c_int * 3)(*dims)
    for call in range(2):
        out = N.fr_stats()
        rc = lib.fr_stats_noalloc(*(x.data_ptr() for x in t), c_dims, 4, 0.2, C.byref(out), None)
        assert rc == N.FR_OK, lib.fr_last_error(None)
        assert out.folds == os_["folds"], (call, out.folds, os_["folds"])
        assert rel_err(out.e_data, os_["e_data"]) <= 1e-12, call
        assert rel_err(out.e_reg, os_["e_reg"]) <= 1e-12, call
        assert list(out.dice_inter[:4]) == list(os_["dice_inter"][:4]), call
        assert list(out.dice_count[:4]) == list(os_["dice_count"][:4]), call
