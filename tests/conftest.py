import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library on a machine with a GPU; GPU tests fail loudly without it."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test on a machine without CUDA")
    from gpuboscia_gb300 import _abi, build
    build.build()
    return _abi.load()
