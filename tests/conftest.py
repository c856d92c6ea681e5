import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs libmgbf kernels)")


@pytest.fixture(scope="session")
def lib():
    """Build (if needed) and load libmgbf.so."""
    from standalone_mgbf_loc_gb300 import build as b
    b.build()
    from standalone_mgbf_loc_gb300 import _abi
    return _abi.load()


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
