import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: minutes of CPU work for the oracle (full-size checks)")


def _ensure_built():
    from fastreg_gb300 import _native, build as fbuild
    if not _native.LIB_PATH.exists():
        fbuild.build()
    from oracle import build as obuild
    if not (ROOT / "oracle" / "_build" / "libfr_oracle32.so").exists():
        obuild.build()


_ensure_built()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("this test needs a CUDA GPU")
    return torch.device("cuda:0")
