import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_built():
    """Builds the C restatement of the oracle (and the reference harness where
    the reference sources exist)."""
    from oracle import oracle as O
    O.build(reference=True)
    return O


@pytest.fixture(scope="session")
def dvr_lib():
    """Builds and loads libdvr_gb300.so."""
    from diffdvr_gb300 import build, _abi
    build.build()
    return _abi.load()


@pytest.fixture(scope="session")
def cuda_device(dvr_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test requested but CUDA is not available")
    return torch.device("cuda:0")
