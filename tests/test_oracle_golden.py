"""The FP64 oracle (oracle/gauss_oracle.c) against the reference's own outputs.

kernel_precision.npz / kernel_random.npz were produced by the reference's ExactKernel and
AbstractKernel compiled from its sources (tests/golden/make_golden.py). The oracle must reproduce
them to ~1e-12 before it may judge the GPU library.
"""
import os

import numpy as np
import pytest

from tests.conftest import reference_compare
from tests.golden.fixtures import precision_fixture, random_cases

TOL = 1e-11  # FP64 restatement vs FP64 reference (summation order of the Hessian forms differs)


def _ops(port, X, Y, W, Z, sigma, W3, golden, prefix):
    d = X.shape[1]
    checks = 0

    def chk(key, val):
        nonlocal checks
        ref = golden[prefix + key]
        assert reference_compare(ref, val, TOL) <= TOL, key
        checks += 1

    chk("convolve", port.convolve(X, Y, W, sigma))
    chk("grad_varlin", port.grad_varlin(X, Y, W, sigma))
    Za = golden[prefix + "grad_alpha_alpha"]
    chk("grad_alpha", port.grad_alpha(X, Y, W, sigma, Za))
    for dim in range(d):
        chk(f"grad_dim_{dim}", port.grad_dim(Y, Y, W, sigma, dim))
        chk(f"grad_dim_x_{dim}", port.grad_dim(X, Y, W, sigma, dim))
    if prefix + "grad_kdp" in golden:
        chk("grad_kdp", port.grad_kdp(X, Y, W, sigma, W.shape[1] - 1, d - 1))
    else:
        import oracle.kernels
        with pytest.raises(oracle.kernels.OracleError):
            port.grad_kdp(X, Y, W, sigma, W.shape[1] - 1, d - 1)
    chk("hess_full", port.hess_full(X, Y, W, sigma))
    for r in range(d):
        for c in range(d):
            chk(f"hess_rowcol_{r}{c}", port.hess_rowcol(X, Y, W, sigma, r, c))
    chk("hess_kdpdq", port.hess_kdpdq(X, Y, W, sigma, 0, 0, d - 1))
    chk("special_hessian", port.special_hessian(Y, W3, sigma, W3))
    return checks


def test_port_matches_reference_precision_fixture(port, golden_precision):
    fx = precision_fixture()
    n = 0
    for d in (2, 3):
        X, Y, Z, W3 = fx[f"X{d}D"], fx[f"Y{d}D"], fx[f"Z{d}D"], fx[f"W{d}D"]
        for wname in ([f"W{d}D", "W4D"] if d == 2 else [f"W{d}D", "W6D"]):
            n += _ops(port, X, Y, fx[wname], Z, fx["kernel_width"], W3, golden_precision,
                      f"d{d}_{wname}_")
    assert n > 60


def test_port_matches_reference_random_cases(port, golden_random):
    n = 0
    for name, c in random_cases().items():
        n += _ops(port, c["X"], c["Y"], c["W"], c["Z"], c["sigma"], c["W3"], golden_random, name + "_")
    assert n > 60


def test_fixture_quirk_identical_prefix():
    """The reference's fixture re-seeds mt19937(1) per matrix: Y2D, W2D and the first 201 rows
    of X2D are identical (AbstractTestKernelPrecision.cxx:21-29)."""
    fx = precision_fixture()
    assert np.array_equal(fx["Y2D"], fx["W2D"])
    assert np.array_equal(fx["X2D"][:201], fx["Y2D"])
    assert fx["X3D"].min() >= np.exp(-1) and fx["X3D"].max() <= 1.0


def test_port_against_live_reference():
    """When the reference tree is present, compare the port with the compiled reference live."""
    import oracle
    if not os.path.exists(oracle.reference_path()) and oracle.build_reference() is None:
        pytest.skip("reference tree not available")
    ref = oracle.load("reference")
    port = oracle.load("port")
    rng = np.random.default_rng(99)
    X, Y = rng.random((123, 3)), rng.random((77, 3))
    W, A = rng.standard_normal((77, 3)), rng.standard_normal((123, 3))
    for a, b in [(ref.convolve(X, Y, W, 0.15), port.convolve(X, Y, W, 0.15)),
                 (ref.grad_alpha(X, Y, W, 0.15, A), port.grad_alpha(X, Y, W, 0.15, A)),
                 (ref.special_hessian(Y, W, 0.15, W[::-1].copy()), port.special_hessian(Y, W, 0.15, W[::-1].copy()))]:
        assert reference_compare(a, b, TOL) <= TOL


def test_source_side_adjoint_by_symmetry(port):
    """gy, gw of the fused adjoint equal finite differences of L = sum alpha . (K W)."""
    rng = np.random.default_rng(5)
    X, Y = rng.random((9, 3)), rng.random((7, 3))
    W, A = rng.standard_normal((7, 3)), rng.standard_normal((9, 3))
    s = 0.4
    v, gx, gy, gw = port.fwd_adjoint(X, Y, W, s, A)
    L = lambda X_, Y_, W_: float(np.sum(A * port.convolve(X_, Y_, W_, s)))
    eps = 1e-6
    for M, g, which in [(X, gx, 0), (Y, gy, 1), (W, gw, 2)]:
        fd = np.zeros_like(M)
        for idx in np.ndindex(M.shape):
            P, N = M.copy(), M.copy()
            P[idx] += eps
            N[idx] -= eps
            args_p = [X, Y, W]
            args_n = [X, Y, W]
            args_p[which], args_n[which] = P, N
            fd[idx] = (L(*args_p) - L(*args_n)) / (2 * eps)
        assert np.max(np.abs(fd - g)) < 1e-6 * max(1.0, np.max(np.abs(g)))
