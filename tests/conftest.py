import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as ge  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine through the C ABI")


def cuda_available():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def pkg():
    return ge.load_package()


@pytest.fixture(scope="session")
def orc():
    o = ge.load_oracle()
    o.build()
    return o


@pytest.fixture(scope="session")
def engine_lib(pkg):
    """The built engine library; on a GPU run a missing CUDA device is an error, not a skip."""
    if not cuda_available():
        pytest.fail("no CUDA device visible for a gpu-marked test")
    pkg.build_lib.build()
    return pkg.engine.load()
