"""The command-line app and the NIfTI codec without a GPU."""
import subprocess

import numpy as np
import pytest

from fastreg_gb300 import _native as N, nifti
from tests.test_abi_host import REFERENCE_INI

APP = N.LIB_PATH.parent / "fastreg_app"


def test_nifti_round_trip(tmp_path):
    r = np.random.Generator(np.random.PCG64(0))
    img = r.normal(0, 1, (5, 6, 7)).astype(np.float32)
    lab = r.integers(0, 9, (5, 6, 7)).astype(np.int16)
    nifti.write(tmp_path / "i.nii", img)
    nifti.write(tmp_path / "l.nii", lab)
    assert np.array_equal(nifti.read(tmp_path / "i.nii"), img)
    assert np.array_equal(nifti.read(tmp_path / "l.nii"), lab)


def test_app_help_and_errors(tmp_path):
    out = subprocess.run([str(APP), "--help"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0 and "USAGE" in out.stdout
    out = subprocess.run([str(APP), "a", "b"], capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "incorrect number of arguments" in out.stderr
    ini = tmp_path / "params.ini"
    ini.write_text(REFERENCE_INI)
    out = subprocess.run([str(APP), str(ini), str(tmp_path / "missing.nii"), "b", "c", "d", str(tmp_path)],
                         capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "cannot open" in out.stderr


def test_app_without_gpu_fails_cleanly(tmp_path):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ini = tmp_path / "params.ini"
    ini.write_text(REFERENCE_INI)
    vol = np.zeros((6, 6, 6), np.float32)
    lab = np.zeros((6, 6, 6), np.int16)
    for n, v in (("t.nii", vol), ("tl.nii", lab), ("s.nii", vol), ("sl.nii", lab)):
        nifti.write(tmp_path / n, v)
    out = subprocess.run([str(APP), str(ini), *(str(tmp_path / n) for n in ("t.nii", "tl.nii", "s.nii", "sl.nii")),
                          str(tmp_path)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 1 and "error" in out.stderr
