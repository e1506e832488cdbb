"""Test configuration: the ``gpu`` marker and import paths.

CPU tests (``-m "not gpu"``) cover the oracle, the host logic and the C-ABI
exports; ``-m gpu`` tests call the CUDA library through the C ABI and compare
it with the oracle.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "modpath-rw_gb300"
for p in (str(PKG), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmprw_gpu.so")


@pytest.fixture(scope="session")
def gpu_lib():
    """Build (if stale) and load the CUDA library; skip nothing -- a GPU test
    without a GPU is an error, not a skip."""
    import torch
    from mprw import build as B
    B.build()
    import mprw
    assert torch.cuda.is_available(), "gpu test collected on a machine without CUDA"
    return mprw.load_library()
