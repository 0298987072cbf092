"""The image-grid oracle (oracle/image.py): pixel order, the windowed sum of
ExactKernel::ConvolveImageFast against a pair-by-pair restatement, its truncation against the exact
sum, the rounding of the window start, and the image-map flow's special cases. The reference has no
test of this path (it needs ITK); ConvolveImageFast and both ConvolveGradientImageFast overloads are
pinned against the reference's own compiled code run on ITK stand-ins with ITK's documented index,
crop and iteration behaviour (tests/golden/image_fast.npz, tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import image as IM


def test_image_points_first_index_fastest():
    pts = IM.image_points([1.0, -2.0, 0.5], [0.5, 1.0, 2.0], [3, 2, 2])
    rows = []
    for k in range(2):
        for j in range(2):
            for i in range(3):
                rows.append([1.0 + 0.5 * i, -2.0 + j, 0.5 + 2.0 * k])
    np.testing.assert_array_equal(pts, np.array(rows))


def test_window_start_rounds_half_up():
    sigma = 1.0  # window 6 pixels, start at the index of y - 3
    y = np.array([[6.5, 2.5], [-0.5, 3.0]])
    start, L, lo, hi, ok = IM.windows(y, sigma, [0.0, 0.0], [1.0, 1.0], [10, 10])
    assert L == 6
    np.testing.assert_array_equal(start, [[4, 0], [-3, 0]])
    np.testing.assert_array_equal(lo, [[4, 0], [0, 0]])
    np.testing.assert_array_equal(hi, [[10, 6], [3, 6]])
    assert ok.all()


def _pairwise(x, y, w, sigma, origin, spacing, size):
    """Pair-by-pair: pixel p takes control point j iff its index lies in j's window."""
    d = len(size)
    start, L, _, _, ok = IM.windows(y, sigma, origin, spacing, size)
    assert ok.all()
    idx = np.indices(tuple(size[::-1])).reshape(d, -1)[::-1].T
    V = np.zeros((x.shape[0], d))
    for j in range(y.shape[0]):
        for p in range(x.shape[0]):
            if np.all((idx[p] >= start[j]) & (idx[p] < start[j] + L)):
                sq = 0.0
                for k in range(d):
                    diff = x[p, k] - y[j, k]
                    sq += diff * diff
                V[p] += w[j] * np.exp(-sq / (sigma * sigma))
    return V


@pytest.mark.parametrize("d", [2, 3])
def test_convolve_image_fast_matches_pairwise(d):
    rng = np.random.default_rng(4 + d)
    size = [9, 7, 5][:d]
    origin, spacing = rng.normal(size=d), rng.uniform(0.5, 1.5, size=d)
    pts = IM.image_points(origin, spacing, size)
    x = pts + 0.1 * rng.normal(size=pts.shape)
    y = origin + spacing * rng.uniform(0, 1, size=(6, d)) * (np.array(size) - 1)
    w = rng.normal(size=(6, d))
    sigma = 0.9
    got = IM.convolve_image_fast(x, y, w, sigma, origin, spacing, size)
    ref = _pairwise(x, y, w, sigma, origin, spacing, size)
    np.testing.assert_allclose(got, ref, rtol=1e-14, atol=1e-15)


def test_window_truncation_against_exact_sum():
    """Unit spacing and control points well inside: the window holds +-3 sigma, so the windowed sum
    is the exact sum up to the Gaussian's tails."""
    rng = np.random.default_rng(2)
    size, sigma = [40, 40], 3.0
    pts = IM.image_points([0.0, 0.0], [1.0, 1.0], size)
    y = rng.uniform(12, 28, size=(10, 2))
    w = rng.normal(size=(10, 2))
    got = IM.convolve_image_fast(pts, y, w, sigma, [0.0, 0.0], [1.0, 1.0], size)
    ex = IM._exact_convolve(pts, y, w, sigma)
    assert np.linalg.norm(got - ex) <= 2e-2 * np.linalg.norm(ex)


def test_window_missing_the_image_raises():
    x = IM.image_points([0.0, 0.0], [1.0, 1.0], [8, 8])
    with pytest.raises(ValueError):
        IM.convolve_image_fast(x, np.array([[40.0, 3.0]]), np.ones((1, 2)), 1.0, [0.0, 0.0], [1.0, 1.0], [8, 8])
    with pytest.raises(ValueError):
        IM.convolve_image_fast(x[:10], np.array([[3.0, 3.0]]), np.ones((1, 2)), 1.0, [0.0, 0.0], [1.0, 1.0], [8, 8])


def test_flow_image_maps_special_cases():
    rng = np.random.default_rng(9)
    size, T = [12, 10], 5
    pos = np.repeat(rng.uniform(3, 8, size=(1, 4, 2)), T, axis=0)
    pts = IM.image_points([0.0, 0.0], [1.0, 1.0], size)
    maps, stop = IM.flow_image_maps(pos, np.zeros_like(pos), 1.5, [0.0, 0.0], [1.0, 1.0], size)
    assert stop is None and np.all(maps == pts[None])
    mom = rng.normal(size=pos.shape)
    maps, stop = IM.flow_image_maps(pos, mom, 1.5, [0.0, 0.0], [1.0, 1.0], size, heun=False)
    dY = IM.convolve_image_fast(pts, pos[T - 1], mom[T - 1], 1.5, [0.0, 0.0], [1.0, 1.0], size)
    np.testing.assert_array_equal(maps[T - 2], pts - dY * (1.0 / (T - 1)))
    np.testing.assert_array_equal(maps[T - 1], pts)
    # a box the first step leaves: stop at T-2, the earlier maps stay the image points
    box = np.array([[0.0, 11.0], [0.0, 9.0]])
    maps, stop = IM.flow_image_maps(pos, 5 * mom, 1.5, [0.0, 0.0], [1.0, 1.0], size, bbox=box)
    assert stop == T - 2
    assert np.all(maps[: T - 2] == pts[None])


def test_bench_window_count_matches_the_restatement():
    """bench.py counts window pairs without the oracle; the count equals the restatement's windows."""
    n, sigma = 40, 2.5
    rng = np.random.default_rng(13)
    origin, spacing = np.array([0.5, -1.0, 2.0]), np.array([1.0, 0.8, 1.2])
    cp = origin + spacing * rng.uniform(-5, n + 5, size=(60, 3))
    import bench
    _, L, lo, hi, _ = IM.windows(cp, sigma, origin, spacing, [n] * 3)
    ref = np.prod(np.maximum(hi - lo, 0), axis=1).sum()
    assert bench.image_window_pairs(cp, sigma, origin, spacing, [n] * 3) == ref


GOLDEN_CASES = ("d2", "d2w4", "d3", "d3w4")


@pytest.fixture(scope="module")
def image_golden():
    import os
    from tests.conftest import GOLDEN
    return dict(np.load(os.path.join(GOLDEN, "image_fast.npz")))


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_restatement_matches_the_reference_image_methods(image_golden, name):
    """ConvolveImageFast and both ConvolveGradientImageFast overloads of the reference (golden
    vectors from its compiled ExactKernel) against the restatement, to FP64 rounding."""
    g = {k[len(name) + 1:]: v for k, v in image_golden.items() if k.startswith(name + "_")}
    args = (g["x"], g["y"], g["w"], float(g["sigma"]), g["origin"], g["spacing"], [int(v) for v in g["size"]])
    if "convolve" in g:
        v = IM.convolve_image_fast(*args)
        assert np.abs(v - g["convolve"]).max() <= 1e-14 * np.abs(g["convolve"]).max()
    G = IM.convolve_gradient_image_fast(*args)
    assert G.shape == g["gradient"].shape
    assert np.abs(G - g["gradient"]).max() <= 1e-14 * np.abs(g["gradient"]).max()
    assert (g["gradient"] == 0).any() and (g["gradient"] != 0).mean() > 0.5  # cropped and covered pixels
    H = IM.convolve_gradient_image_fast(*args, alpha=g["alpha"])
    assert np.abs(H - g["gradient_alpha"]).max() <= 1e-14 * np.abs(g["gradient_alpha"]).max()


def test_image_gradient_is_the_derivative_of_the_windowed_sum():
    """Inside every window, d/dx_p of sum_j W_jk K(x_p, y_j) is the gradient's row (finite
    differences on one pixel's coordinates; the windows do not move with x)."""
    rng = np.random.default_rng(3)
    size, origin, spacing, sigma = [12, 10], [0.0, 0.0], [1.0, 1.0], 1.6
    x = IM.image_points(origin, spacing, size)
    y = rng.uniform([2, 2], [9, 7], (5, 2))
    w = rng.standard_normal((5, 2))
    G = IM.convolve_gradient_image_fast(x, y, w, sigma, origin, spacing, size)
    p, eps = 47, 1e-6
    for l in range(2):
        xp, xm = x.copy(), x.copy()
        xp[p, l] += eps
        xm[p, l] -= eps
        fd = (IM.convolve_image_fast(xp, y, w, sigma, origin, spacing, size)[p]
              - IM.convolve_image_fast(xm, y, w, sigma, origin, spacing, size)[p]) / (2 * eps)
        np.testing.assert_allclose(G[p, :, l], fd, rtol=1e-6, atol=1e-9)
