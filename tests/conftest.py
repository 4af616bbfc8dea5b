import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA device (GB300); parity of the GPU "
        "library against the oracle and the reference's golden vectors")


@pytest.fixture(scope="session")
def oracle_lib():
    from miniamr_gb300 import build
    from miniamr_gb300.abi import Library
    return Library(build.build_oracle())


@pytest.fixture(scope="session")
def gpu_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("gpu test without a CUDA device")
    from miniamr_gb300 import build, load
    build.build_library()
    return load()
