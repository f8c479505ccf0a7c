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
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def ctx():
    """One lj_gpu context for the GPU tests (built in-tree, never a fallback)."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    torch.cuda.init()
    from lajolla_public_gb300 import gpu
    c = gpu.Context(0)
    yield c
    c.close()
