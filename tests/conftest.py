import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def dd():
    import __graft_entry__
    return __graft_entry__.load_package()


@pytest.fixture(scope="session")
def cuda(dd):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")
