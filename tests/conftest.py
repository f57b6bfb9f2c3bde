"""Shared fixtures. `gpu` marks tests that need a CUDA device (run on a GB300
with `pytest -m gpu`); everything else runs on any CPU host."""
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = Path(__file__).resolve().parent / "golden"
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (sm_103a build of the library)")
    config.addinivalue_line("markers", "slow: long-running")


def golden(name: str):
    return np.load(GOLDEN / f"{name}.npz")


@pytest.fixture(scope="session")
def orc():
    import oracle

    return oracle.Oracle()


@pytest.fixture(scope="session")
def ref():
    import oracle

    if not oracle.REF_SO.exists():
        pytest.skip("oracle/_ref not built (needs the reference source tree)")
    return oracle.Reference()


@pytest.fixture(scope="session")
def lib():
    """The CUDA library on a GPU host; fails loudly if it is missing there."""
    import aleator_gb300 as A

    A.load_library()
    info = A.device_info()
    return A, info


def rel_err(a, b, floor=1.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(floor, np.abs(b))
