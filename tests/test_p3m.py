"""The particle-mesh (P3M) oracle (oracle/p3m.py, a restatement of the reference's P3MKernel): the
grid rule, the approximation error against the exact kernel (within the 8e-2 the reference's tests
accept for P3M), and every method against the reference's own P3MKernel compiled from its source on
ITK stand-ins (direct DFTs in place of VNL's FFT; tests/golden/p3m_reference.npz, made by
tests/golden/make_golden.py). No GPU."""
import os

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


P3M_GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "p3m_reference.npz")
P3M_CASES = ("d2", "d2out", "d3", "d3dv2")


def p3m_case(name):
    z = np.load(P3M_GOLDEN)
    return {k[len(name) + 1:]: z[k] for k in z.files if k.startswith(name + "_")}


def p3m_restated(c):
    """Every P3MKernel method of the restatement on one golden case (keys as in the fixture)."""
    from oracle import p3m
    x, y, w, sigma = c["x"], c["y"], c["w"], float(c["sigma"])
    d = x.shape[1]
    kw = dict(lo=c["lo"], hi=c["hi"], ratio=float(c["ratio"]), padding=float(c["padding"]))
    return {
        "convolve": p3m.convolve(x, y, w, sigma, **kw),
        "gradient": p3m.convolve_gradient(x, y, w, sigma, **kw),
        "gradient_alpha": p3m.convolve_gradient_alpha(x, y, w, sigma, c["alpha"], **kw),
        "gradient_dim": p3m.convolve_gradient_dim(x, y, w, sigma, d - 1, **kw),
        "hessian": p3m.convolve_hessian(x, y, w, sigma, **kw),
        "hessian_rowcol": p3m.convolve_hessian_rowcol(x, y, w, sigma, d - 1, 0, **kw),
        "special_hessian": p3m.special_hessian(c["ys"], c["beta"], sigma, c["xi"], c["ys_lo"], c["ys_hi"],
                                               float(c["ratio"]), float(c["padding"])),
    }


@pytest.mark.parametrize("name", P3M_CASES)
def test_restatement_matches_the_reference_p3m(name):
    """The FP64 restatement reproduces the reference's P3MKernel (every overload, the special Hessian
    composed over its Hessians, points outside the data domain) to rounding: the two differ only in
    the order of the transform sums."""
    c = p3m_case(name)
    for key, got in p3m_restated(c).items():
        ref = c[key]
        assert got.shape == ref.shape, key
        assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref), key
    if name == "d2out":  # targets off the grid get nothing, in the reference as in the restatement
        assert np.count_nonzero(np.all(c["convolve"] == 0, axis=1)) > 0


def test_reference_p3m_library_matches_its_golden_vectors():
    """Where the reference tree is present, its P3MKernel built on the stand-ins still gives the
    committed vectors (the fixture is current)."""
    import oracle
    if oracle.build_reference() is None:
        pytest.skip("reference tree absent")
    ref = oracle.load("reference")
    c = p3m_case("d3dv2")
    got = ref.p3m("gradient_alpha", c["x"], c["y"], c["w"], float(c["sigma"]), c["lo"], c["hi"],
                  float(c["ratio"]), float(c["padding"]), alpha=c["alpha"])
    assert np.array_equal(got, c["gradient_alpha"])
