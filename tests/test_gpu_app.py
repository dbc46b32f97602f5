"""The command-line app end to end on the GPU: NIfTI in, NIfTI out, the same bits as the
library called directly."""
import subprocess

import numpy as np
import pytest

from fastreg_gb300 import FastReg, Params, _native as N, nifti
from tests.helpers import images

pytestmark = pytest.mark.gpu
APP = N.LIB_PATH.parent / "fastreg_app"


def test_app_registers_nifti_volumes(cuda, tmp_path):
    import torch
    dims = (24, 20, 18)
    d = images(dims, 31)
    ini = tmp_path / "params.ini"
    ini.write_text("NO_LABELS=4\nMAX_ITER=40\nALPHA=0.02\nTAU=0.2\nW_REG=0.2\nRHO_0=1.0\np=2.0\nC=0.25\n"
                   "MAX_UPDATE_NORM=-1e-10\nRESET_ITER=-1\n")
    for n, k in (("target.nii", "T"), ("target_labels.nii", "labT"), ("source.nii", "S"),
                 ("source_labels.nii", "labS")):
        nifti.write(tmp_path / n, d[k])
    out_dir = tmp_path / "out"
    out_dir.mkdir()
    r = subprocess.run([str(APP), str(ini), *(str(tmp_path / n) for n in ("target.nii", "target_labels.nii",
                                                                          "source.nii", "source_labels.nii")),
                        str(out_dir)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert "REGISTRATION TIME" in r.stdout and "SAVED OUTPUT" in r.stdout

    P = Params(volume_dims=dims, no_labels=4, max_iter=40, alpha=0.02)
    fr = FastReg(P)
    bufs = [torch.from_numpy(d[k]).to(cuda) for k in ("T", "labT", "S", "labS")]
    fr(*bufs)
    name = "source.nii"
    expect = {f"target_psi_inv_{name}.nii": bufs[0], f"source_psi_{name}.nii": bufs[2],
              f"target_psi_inv_labels_{name}.nii": bufs[1], f"source_psi_labels_{name}.nii": bufs[3]}
    for fn, t in expect.items():
        got = nifti.read(out_dir / fn)
        assert np.array_equal(got, t.cpu().numpy()), fn
