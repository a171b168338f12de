"""Shared pytest configuration: the `gpu` marker and helpers used by several test files."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_vectors.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


def rel_l2(a, b) -> float:
    """||a - b|| / ||b||, in float64 (b is the reference)."""
    a = np.asarray(a).astype(np.complex128 if np.iscomplexobj(a) else np.float64).ravel()
    b = np.asarray(b).astype(np.complex128 if np.iscomplexobj(b) else np.float64).ravel()
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    return float(num / den) if den else float(num)
