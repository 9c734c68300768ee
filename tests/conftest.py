"""Shared test setup: the `gpu` marker, library/oracle builds, helpers."""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

ALL_DTYPES = [np.int8, np.uint8, np.int16, np.uint16, np.int32, np.uint32, np.int64, np.uint64]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300 box)")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def native_lib():
    """The in-tree libturtle_gb300.so (built if missing)."""
    from turtlesort_gb300 import build as b
    b.build()
    import turtlesort_gb300
    return turtlesort_gb300.load_library()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu(native_lib):
    if not has_gpu():
        pytest.skip("no CUDA device")
    return native_lib
