import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds (if needed) and loads the native library and the oracle."""
    from network_relaxation_gb300 import build as nbuild

    nbuild.build()
    import oracle

    oracle.build()
    import network_relaxation_gb300 as nr

    return nr.lib()


@pytest.fixture(scope="session")
def cuda(built):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test scheduled on a machine without CUDA")
    torch.cuda.init()
    return torch.device("cuda:0")
