"""The particle-mesh (P3M) oracle (oracle/p3m.py, a restatement of the reference's P3MKernel,
whose own build needs ITK/FFTW): the grid rule and the approximation error against the exact
kernel, within the 8e-2 the reference's tests accept for P3M. No GPU."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def K():
    import oracle
    return oracle.load("port")


def test_grid_rule():
    from oracle import p3m
    origin, size, s = p3m.grid([0.0, 0.0, 0.0], [1.0, 1.0, 1.0], 0.1)
    assert s == pytest.approx(0.02) and list(size) == [128, 128, 128]  # 1.6 / 0.02 = 80 -> 128
    assert origin[0] == pytest.approx(-(128 * 0.02 - 1.0) / 2)
    origin, size, s = p3m.grid([0.0, -1.0], [2.0, 1.0], 0.5, ratio=0.25, padding=1.0)
    assert list(size) == [32, 32]  # (2 + 1) / 0.125 = 24 -> 32


@pytest.mark.parametrize("d,sigma", [(2, 0.1), (2, 0.3), (3, 0.3)])
def test_approximation_error(K, d, sigma):
    from oracle import p3m
    rng = np.random.default_rng(7 + d)
    x, y = rng.random((120, d)), rng.random((150, d))
    w, a = rng.normal(size=(150, 3)), rng.normal(size=(120, 3))
    v, ve = p3m.convolve(x, y, w, sigma), K.convolve(x, y, w, sigma)
    g, ge = p3m.convolve_gradient_alpha(x, y, w, sigma, a), K.grad_alpha(x, y, w, sigma, a)
    assert np.linalg.norm(v - ve) <= 8e-2 * np.linalg.norm(ve)
    assert np.linalg.norm(g - ge) <= 8e-2 * np.linalg.norm(ge)
    gv = p3m.convolve_gradient(x, y, w, sigma)
    np.testing.assert_allclose(np.einsum("ikp,ik->ip", gv, a), g, rtol=1e-12, atol=1e-12)


def test_gradient_dim_and_hessian_restatements():
    """P3MKernel::ConvolveGradient(X, dim) is the dim column of ConvolveGradient(X); ConvolveHessian(X)
    is symmetric and its (row, col) entry is ConvolveHessian(X, row, col); both within the
    reference's 8e-2 of the exact sums."""
    import oracle
    from oracle import p3m
    K = oracle.load("port")
    rng = np.random.default_rng(8)
    x, y, w = rng.random((60, 3)), rng.random((70, 3)), rng.normal(size=(70, 2))
    g = p3m.convolve_gradient(x, y, w, 0.3)
    for dim in range(3):
        assert np.array_equal(p3m.convolve_gradient_dim(x, y, w, 0.3, dim), g[:, :, dim])
    h = p3m.convolve_hessian(x, y, w, 0.3)
    assert np.array_equal(h, np.swapaxes(h, 2, 3))
    assert np.array_equal(p3m.convolve_hessian_rowcol(x, y, w, 0.3, 2, 1), h[:, :, 1, 2])
    he = np.asarray(K.hess_full(x, y, w, 0.3)).reshape(h.shape)
    assert np.linalg.norm(h - he) <= 8e-2 * np.linalg.norm(he)
    ge = np.asarray(K.grad_dim(x, y, w, 0.3, 1)).reshape(60, 2)
    assert np.linalg.norm(g[:, :, 1] - ge) <= 8e-2 * np.linalg.norm(ge)


def test_special_hessian_composition():
    """AbstractKernel::ConvolveSpecialHessian composed from the P3M Hessians (as P3MKernel inherits
    it) stays within the reference's 8e-2 of the exact special Hessian."""
    import oracle
    from oracle import p3m
    K = oracle.load("port")
    rng = np.random.default_rng(3)
    y, b, xi = rng.random((80, 3)), rng.normal(size=(80, 3)), rng.normal(size=(80, 3))
    sh = p3m.special_hessian(y, b, 0.3, xi)
    ex = np.asarray(K.special_hessian(y, b, 0.3, xi)).reshape(sh.shape)
    assert np.linalg.norm(sh - ex) <= 8e-2 * np.linalg.norm(ex)


def test_bench_grid_rule_matches_the_restatement():
    import bench
    from oracle import p3m
    rng = np.random.default_rng(12)
    for _ in range(20):
        d = int(rng.integers(2, 4))
        lo = rng.normal(size=d)
        hi = lo + rng.uniform(0.1, 3.0, size=d)
        sigma, ratio = float(rng.uniform(0.03, 0.5)), float(rng.choice([0.1, 0.2, 0.3, 0.5]))
        assert bench.p3m_grid_size(lo, hi, sigma, ratio) == [int(v) for v in p3m.grid(lo, hi, sigma, ratio)[1]]
