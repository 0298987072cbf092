"""Deterministic test inputs shared by the fixture generator and the tests.

``precision_fixture`` reproduces AbstractTestKernelPrecision (tests/unit_tests/kernels/
AbstractTestKernelPrecision.h:22-60 and .cxx:21-29 of the reference): kernel width 1.88,
X 501 rows, Y 201 rows, W 201 rows, Z 501 rows, entries exp(-gen()/gen.max()) where
``std::mt19937 gen(1)`` is re-seeded for every matrix and filled row by row. numpy's legacy
MT19937 seeding with an integer is the same generator as std::mt19937(seed).
"""
from __future__ import annotations

import numpy as np

_MT_MAX = 4294967295.0


def mt19937_matrix(rows: int, cols: int) -> np.ndarray:
    bg = np.random.MT19937(0)
    bg._legacy_seeding(1)
    raw = bg.random_raw(rows * cols).astype(np.float64)
    return np.exp(-raw / _MT_MAX).reshape(rows, cols)


def precision_fixture() -> dict:
    X_ROW, Y_ROW = 501, 201
    fx = {"kernel_width": 1.88}
    for d in (2, 3):
        fx[f"X{d}D"] = mt19937_matrix(X_ROW, d)
        fx[f"Y{d}D"] = mt19937_matrix(Y_ROW, d)
        fx[f"W{d}D"] = mt19937_matrix(Y_ROW, d)
        fx[f"Z{d}D"] = mt19937_matrix(X_ROW, d)
    fx["W4D"] = mt19937_matrix(Y_ROW, 4)
    fx["W6D"] = mt19937_matrix(Y_ROW, 6)
    return fx


def random_cases() -> dict:
    """Non-degenerate, ragged cases: uniform points, N(0,1) weights (K spans many decades)."""
    cases = {}
    specs = [
        ("r3a", 3, 3, 300, 257, 0.2, 11),
        ("r3b", 3, 6, 193, 97, 0.05, 12),
        ("r3c", 3, 5, 65, 300, 0.3, 13),  # dv = 5: column chunks
        ("r2a", 2, 2, 257, 300, 0.1, 14),
        ("r2b", 2, 4, 31, 129, 0.25, 15),
    ]
    for name, d, dv, nx, ny, sigma, seed in specs:
        rng = np.random.default_rng(seed)
        cases[name] = {
            "X": rng.random((nx, d)),
            "Y": rng.random((ny, d)),
            "W": rng.standard_normal((ny, dv)),
            "Z": rng.standard_normal((nx, max(dv, d))),
            "W3": rng.standard_normal((ny, d)),
            "sigma": sigma,
        }
    return cases
