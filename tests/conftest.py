import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built native library")


@pytest.fixture(scope="session")
def native_lib():
    from fluxcore3d_gb300 import _build, _lib
    _build.build()
    return _lib.lib()


@pytest.fixture(scope="session")
def cuda(native_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    return torch.device("cuda")
