"""Shared pytest configuration.

Markers: ``gpu`` marks tests that need a CUDA device (run with ``-m gpu``).
The package directory (periodic-lbm_gb300/) and the repository root are put
on sys.path so that ``import plbm`` and ``import oracle.oracle`` work.
"""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "periodic-lbm_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU and libplbmgpu.so")


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(ROOT / "tests" / "golden" / "golden.npz"))


@pytest.fixture(scope="session")
def gpu_lib():
    """libplbmgpu.so, built if needed; fails loudly if it cannot be loaded."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a gpu-marked test ran without a visible CUDA device")
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    ge.build()
    from plbm import _lib
    return _lib.load()
