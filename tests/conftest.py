"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU.

The oracle (oracle/, test infrastructure only) is built on first use.
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from pyoracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if needed) and loads the CUDA library; skips nothing -- a GPU
    test must run the native path."""
    import torch
    assert torch.cuda.is_available(), "GPU test without a GPU"
    from epetreco_gb300 import build
    build.build()
    from epetreco_gb300 import _lib
    return _lib.lib()
