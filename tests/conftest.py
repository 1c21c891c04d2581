"""Shared test setup: the `gpu` marker, the repo root on sys.path, and fixtures for
the package (imported by its directory name) and the CPU oracle."""
from __future__ import annotations

import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_package():
    return importlib.import_module("shallow-water_gb300")


@pytest.fixture(scope="session")
def sw():
    return load_package()


@pytest.fixture(scope="session")
def port():
    from oracle import port as p
    p.build()
    return p


@pytest.fixture(scope="session")
def problems(sw):
    return sw.problems


@pytest.fixture(scope="session")
def gpu_lib(sw):
    """The built C ABI library on a machine with a GPU; the test fails (not skips) if the
    library is missing, so a GPU run can never pass on a fallback."""
    import torch  # noqa: F401  (plumbing: confirms the CUDA runtime sees a device)
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return sw.lib()


def bitwise_equal(a: np.ndarray, b: np.ndarray) -> bool:
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def max_rel_err(a: np.ndarray, b: np.ndarray) -> float:
    """max |a - b| / max |b| over the interior (normwise relative error)."""
    ai, bi = a[2:-2, 2:-2], b[2:-2, 2:-2]
    scale = float(np.abs(bi).max())
    return float(np.abs(ai - bi).max()) / (scale if scale > 0 else 1.0)
