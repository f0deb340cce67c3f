"""Test configuration: the ``gpu`` marker and import paths.

``-m "not gpu"`` runs on any host (oracle vs golden vectors, host logic,
library loading); ``-m gpu`` needs a CUDA device and the built library.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mb-rec-msot_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built CUDA library")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "mex_golden.npz")))


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from msot_gb300 import _lib
    _lib.load(build_if_missing=True)
    return torch
