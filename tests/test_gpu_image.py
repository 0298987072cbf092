"""GPU image-grid path (gbk_image_points, gbk_convolve_image_fast, gbk_convolve_gradient_image_fast(_alpha),
gbk_flow_image_maps) against the oracle's restatement of ExactKernel::ConvolveImageFast,
ConvolveGradientImageFast and Diffeos' image-map integration (oracle/image.py), and against the
reference's own ExactKernel image methods (golden vectors, tests/golden/image_fast.npz). In GBK_MODE_F64 the windowed sums follow the reference's arithmetic and order of
additions per pixel and differ from the oracle only through exp (1e-13 normwise); GBK_MODE_F32C
evaluates them in FP32 with compensated sums (1e-6)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import deformetrica_code_gb300 as g
    return g


def _case(d, seed=0, ncp=40, T=6):
    rng = np.random.default_rng(seed + d)
    size = [24, 20, 16][:d]
    origin, spacing = rng.normal(size=d), rng.uniform(0.6, 1.4, size=d)
    ext = spacing * (np.array(size) - 1)
    cp = origin + ext * rng.uniform(0.15, 0.85, size=(ncp, d))
    pos = np.stack([cp + 0.2 * t * np.sin(cp + t) for t in range(T)])
    mom = rng.normal(size=(T, ncp, d))
    return size, origin, spacing, pos, mom


def _nrm(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("d", [2, 3])
def test_image_points(gb, d):
    from oracle import image as IM
    size, origin, spacing, _, _ = _case(d)
    im = gb.ImageGrid(origin, spacing, size)
    np.testing.assert_array_equal(im.points(), IM.image_points(origin, spacing, size))


@pytest.mark.parametrize("d,sigma,mode,tol", [(2, 1.7, "F64", 1e-13), (3, 1.2, "F64", 1e-13), (3, 2.5, "F64", 1e-13),
                                               (2, 1.7, "F32C", 1e-6), (3, 2.5, "F32C", 1e-6)])
def test_convolve_image_fast(gb, d, sigma, mode, tol):
    """FP64: the reference's arithmetic (differences from the oracle through exp only); FP32C:
    FP32 exponentials with compensated sums."""
    import torch
    from oracle import image as IM
    size, origin, spacing, pos, mom = _case(d)
    im = gb.ImageGrid(origin, spacing, size)
    rng = np.random.default_rng(3)
    x = IM.image_points(origin, spacing, size) + 0.2 * rng.normal(size=(im.pixels, d))
    ref = IM.convolve_image_fast(x, pos[0], mom[0], sigma, origin, spacing, size)
    k = gb.GB300ExactKernel(d, sigma, mode=getattr(gb, f"GBK_MODE_{mode}"))
    k.SetSources(pos[0])
    k.SetWeights(mom[0])
    got = k.ConvolveImageFast(x, im)
    assert _nrm(got, ref) <= tol
    kd = gb.GB300ExactKernel(d, sigma, context=k.ctx)
    kd.SetSources(torch.from_numpy(pos[0]).cuda())
    kd.SetWeights(torch.from_numpy(mom[0]).cuda())
    got_dev = kd.ConvolveImageFast(torch.from_numpy(x).cuda(), im).cpu().numpy()
    np.testing.assert_array_equal(got_dev, got)


def test_convolve_image_fast_errors(gb):
    size, origin, spacing, pos, mom = _case(2)
    im = gb.ImageGrid(origin, spacing, size)
    x = im.points()
    k = gb.GB300ExactKernel(2, 1.5)
    far = pos[0].copy()
    far[7] += 1000.0
    k.SetSources(far)
    k.SetWeights(mom[0])
    with pytest.raises(gb.GBKError, match="control point 7"):
        k.ConvolveImageFast(x, im)
    k.SetSources(pos[0])
    with pytest.raises(ValueError):
        k.ConvolveImageFast(x[:-1], im)
    k.SetKernelWidth(0.1)  # a window of int(0.6) = 0 pixels
    with pytest.raises(gb.GBKError):
        k.ConvolveImageFast(x, im)


@pytest.mark.parametrize("d,heun", [(2, True), (3, True), (3, False)])
def test_flow_image_maps_fast(gb, d, heun):
    from oracle import image as IM
    size, origin, spacing, pos, mom = _case(d, seed=5)
    sigma = 1.6
    im = gb.ImageGrid(origin, spacing, size)
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    maps, stop = gb.flow_image_maps(pos, 0.3 * mom, sigma, im, heun=heun, fast=True, span=2.0, context=ctx)
    ref, rstop = IM.flow_image_maps(pos, 0.3 * mom, sigma, origin, spacing, size, heun=heun, fast=True, span=2.0)
    assert stop is None and rstop is None
    for t in range(pos.shape[0]):
        assert _nrm(maps[t], ref[t]) <= 1e-13
    np.testing.assert_array_equal(maps[-1], ref[-1])


def test_flow_image_maps_fast_f32c(gb):
    from oracle import image as IM
    size, origin, spacing, pos, mom = _case(3, seed=5)
    im = gb.ImageGrid(origin, spacing, size)
    ctx = gb.Context(mode=gb.GBK_MODE_F32C)
    maps, _ = gb.flow_image_maps(pos, 0.3 * mom, 1.6, im, fast=True, context=ctx)
    ref, _ = IM.flow_image_maps(pos, 0.3 * mom, 1.6, origin, spacing, size, fast=True)
    pts = ref[-1]
    assert np.linalg.norm((maps[0] - pts) - (ref[0] - pts)) <= 1e-6 * np.linalg.norm(ref[0] - pts)


@pytest.mark.parametrize("mode,tol", [("F64", 1e-12), ("F32C", 1e-6)])
def test_flow_image_maps_full_sums(gb, mode, tol):
    from oracle import image as IM
    size, origin, spacing, pos, mom = _case(3, seed=8, ncp=25)
    sigma = 1.6
    im = gb.ImageGrid(origin, spacing, size)
    ctx = gb.Context(mode=getattr(gb, f"GBK_MODE_{mode}"))
    maps, _ = gb.flow_image_maps(pos, 0.3 * mom, sigma, im, fast=False, context=ctx)
    ref, _ = IM.flow_image_maps(pos, 0.3 * mom, sigma, origin, spacing, size, fast=False)
    pts = ref[-1]
    assert np.linalg.norm((maps[0] - pts) - (ref[0] - pts)) <= tol * np.linalg.norm(ref[0] - pts)


def test_flow_image_maps_box_and_zero_momenta(gb):
    from oracle import image as IM
    size, origin, spacing, pos, mom = _case(2, seed=11)
    sigma = 1.6
    im = gb.ImageGrid(origin, spacing, size)
    ext = spacing * (np.array(size) - 1)
    box = np.stack([origin - 0.01 * ext, origin + 1.01 * ext], axis=1)
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    maps, stop = gb.flow_image_maps(pos, 3.0 * mom, sigma, im, bbox=box, context=ctx)
    ref, rstop = IM.flow_image_maps(pos, 3.0 * mom, sigma, origin, spacing, size, bbox=box)
    assert rstop is not None and stop == rstop
    assert _nrm(maps[stop], ref[stop]) <= 1e-13
    np.testing.assert_array_equal(maps[:stop], ref[:stop])
    maps, stop = gb.flow_image_maps(pos, 0.0 * mom, sigma, im, context=ctx)
    assert stop is None
    np.testing.assert_array_equal(maps, np.repeat(im.points()[None], pos.shape[0], axis=0))


GOLDEN_CASES = ("d2", "d2w4", "d3", "d3w4")


@pytest.fixture(scope="module")
def image_golden():
    import os
    from tests.conftest import GOLDEN
    return dict(np.load(os.path.join(GOLDEN, "image_fast.npz")))


def _golden_case(image_golden, name):
    return {k[len(name) + 1:]: v for k, v in image_golden.items() if k.startswith(name + "_")}


@pytest.mark.parametrize("name", GOLDEN_CASES)
@pytest.mark.parametrize("mode,tol", [("F64", 1e-12), ("F32C", 1e-6)])
def test_image_methods_match_the_reference(gb, image_golden, name, mode, tol):
    """ConvolveImageFast and both ConvolveGradientImageFast overloads against the reference's own
    compiled ExactKernel (golden vectors; dv = 4 runs as two column chunks): FP64 to the exp's rounding,
    FP32C normwise within 1e-6; host and device arrays give the same bits."""
    import torch
    g = _golden_case(image_golden, name)
    d = g["x"].shape[1]
    im = gb.ImageGrid(g["origin"], g["spacing"], g["size"])
    k = gb.GB300ExactKernel(d, float(g["sigma"]), mode=getattr(gb, f"GBK_MODE_{mode}"))
    k.SetSources(g["y"])
    k.SetWeights(g["w"])
    got = {"gradient": k.ConvolveGradientImageFast(g["x"], im),
           "gradient_alpha": k.ConvolveGradientImageFast(g["x"], g["alpha"], im)}
    if "convolve" in g:
        got["convolve"] = k.ConvolveImageFast(g["x"], im)
    for key, v in got.items():
        r = g[key].reshape(v.shape[0], -1)
        e = np.linalg.norm(v.reshape(v.shape[0], -1) - r, axis=1).max() / np.linalg.norm(r, axis=1).max()
        assert e <= tol, (key, e)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    kd = gb.GB300ExactKernel(d, float(g["sigma"]), context=k.ctx)
    kd.SetSources(dev(g["y"]))
    kd.SetWeights(dev(g["w"]))
    np.testing.assert_array_equal(kd.ConvolveGradientImageFast(dev(g["x"]), dev(g["alpha"]), im).cpu().numpy(),
                                  got["gradient_alpha"])
    np.testing.assert_array_equal(kd.ConvolveGradientImageFast(dev(g["x"]), im).cpu().numpy(), got["gradient"])


def test_image_gradient_errors(gb):
    size, origin, spacing, pos, mom = _case(2)
    im = gb.ImageGrid(origin, spacing, size)
    k = gb.GB300ExactKernel(2, 1.5)
    k.SetSources(pos[0] + 1e3)  # every window misses the image
    k.SetWeights(mom[0])
    x = im.points()
    with pytest.raises(gb.GBKError, match="misses the image"):
        k.ConvolveGradientImageFast(x, im)
    k.SetSources(pos[0])
    with pytest.raises(RuntimeError, match="count mismatch"):
        k.ConvolveGradientImageFast(x, np.zeros((7, 2)), im)
