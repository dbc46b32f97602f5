"""fr_stats_noalloc: the registration statistics for callers that cannot allocate
device memory (for example a process whose GPU memory is owned by another
framework's pool, or a pipeline that forbids cudaMalloc after start-up).

It must give what fr_get_stats gives after fr_register -- SSD and regulariser
energies within 1e-12 relative (the two reductions add the same per-voxel FP64
terms in different orders), fold count and Dice counts exactly -- on two calls in
a row, since every call reuses the library's one scratch array.  This file is
collected last so that a run stopping at its first failure has run every other
test first."""
import ctypes as C

import numpy as np
import pytest

from fastreg_gb300 import FastReg, Params, _native as N
from tests.helpers import images, rel_err

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
