"""Shared test configuration: the `gpu` marker and helpers to reach the library and the oracle.

Tests marked `gpu` need a CUDA device and call the library through its C ABI; everything else
runs on the CPU (oracle vs golden fixtures, ABI exports, host logic).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def reference_compare(x, y, tol):
    """The reference's element-wise criterion (AbstractTestKernelPrecision.cxx:31-63):
    min(|x - y| / |x|, |x - y|) <= tol for every element; returns the worst value."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    assert x.shape == y.shape, (x.shape, y.shape)
    diff = np.abs(x - y)
    with np.errstate(divide="ignore", invalid="ignore"):
        rel = np.where(x != 0, diff / np.abs(x), np.inf)
    worst = np.minimum(rel, diff)
    return float(worst.max()) if worst.size else 0.0


def normwise_rel(approx, ref):
    """max_i |err_i| / max_i |ref_i| (row norms): relative error of the whole output."""
    a = np.asarray(approx).reshape(np.shape(ref)[0], -1)
    r = np.asarray(ref).reshape(np.shape(ref)[0], -1)
    den = np.linalg.norm(r, axis=1).max()
    if den == 0:
        return float(np.linalg.norm(a - r, axis=1).max())
    return float(np.linalg.norm(a - r, axis=1).max() / den)


@pytest.fixture(scope="session")
def golden_precision():
    return dict(np.load(os.path.join(GOLDEN, "kernel_precision.npz")))


@pytest.fixture(scope="session")
def golden_random():
    return dict(np.load(os.path.join(GOLDEN, "kernel_random.npz")))


@pytest.fixture(scope="session")
def port():
    import oracle
    return oracle.load("port")
