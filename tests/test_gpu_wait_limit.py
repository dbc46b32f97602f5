"""The failure path of the TMA-staged kernels on the GPU, without a fault: a block waits
with their bounded wait on a barrier that nothing completes (fr_selftest_wait_limit), gives
up after the limit (about a second), sets the device error word, and the GPU stays usable
-- a registration right after it gives the oracle's bits."""
import ctypes as C

import numpy as np
import pytest

from fastreg_gb300 import FastReg, Params, _native as N
from oracle import oracle as O
from tests.helpers import assert_bitexact, images

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_context_stays_usable(cuda):
    import torch
    lib = N.load()
    secs = C.c_double()
    rc = lib.fr_selftest_wait_limit(C.byref(secs), None)
    assert rc == N.FR_OK, lib.fr_last_error(None)
    assert 0.3 < secs.value < 30.0, secs.value  # gave up after its limit, not at once, not never
    dims = (20, 18, 16)
    d = images(dims, 3)
    P = Params(volume_dims=dims, no_labels=4, max_iter=10, alpha=0.02, staging=2)
    fr = FastReg(P)
    bufs = [torch.from_numpy(d[k]).to(cuda) for k in ("T", "labT", "S", "labS")]
    fr(*bufs)
    o = O.ref_register(P, d["T"], d["labT"], d["S"], d["labS"])
    assert_bitexact(fr.get_field(N.FR_FIELD_PSI).cpu().numpy(), o["psi"], "psi after the self-test")
    fr.close()
