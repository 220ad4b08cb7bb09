import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built library')


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope='session')
def gpu_lib():
    """The built CUDA library; GPU tests fail (not skip) when it cannot be loaded."""
    from gwfast_gb300 import _build, _lib
    _build.build()
    return _lib.load()
