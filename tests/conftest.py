import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def port():
    import oracle as O
    O.build_port()
    return O.Port()


@pytest.fixture(scope="session")
def cmlib():
    import cardiomechanics_gb300 as cm
    if not cm.LIB_PATH.exists():
        from cardiomechanics_gb300 import build
        build.build()
    cm.lib()
    return cm


@pytest.fixture(scope="session")
def gpu(cmlib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    return cmlib
