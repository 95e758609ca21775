"""Test configuration: the `gpu` marker and shared helpers.

`-m "not gpu"` runs on CPU only: the oracle against the golden vectors, the
host logic, and the C-ABI library load / export checks.  `-m gpu` runs the
parity tests through the C ABI on a GB300.
"""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_collection_modifyitems(config, items):
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    skip = pytest.mark.skip(reason="no CUDA device in this environment")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def native_lib():
    """The built libmpdok_gb300.so (built on demand with nvcc)."""
    from mpdok_gb300 import _build, _native
    if not _native.LIB_PATH.exists():
        _build.build()
    return _native.load()


@pytest.fixture(scope="session")
def golden():
    def load(name):
        return np.load(GOLDEN / f"{name}.npz")
    return load
