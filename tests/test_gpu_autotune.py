"""GPU: the autotuner (gbk_autotune, gbk_autotune_data, gbk_tune_save / gbk_tune_load, GBK_TUNE_FILE).

* It picks a compiled launch shape of the path the call takes (caller order with two-float
  coordinates below the automatic order's size rule, the spatial order above it) and a split count
  within range; the tuned call uses exactly that choice (gbk_last_launch) and still matches the FP64
  oracle.
* Tuning on the caller's data times the spatial path itself (sorts, pruning, bulk staging) and never
  chooses anything slower than the default launch it also times.
* The table survives gbk_tune_save / gbk_tune_load and GBK_TUNE_FILE, with bitwise-equal results; an
  entry from another path's family is ignored (a tuned choice never changes the arithmetic).
"""
import os

import numpy as np
import pytest

from tests.conftest import normwise_rel

pytestmark = pytest.mark.gpu

TWO_FLOAT_FAMILY = {9, 10}
SPATIAL_FAMILY = {11, 12, 0, 1, 2, 3, 4, 8}


@pytest.fixture(scope="module")
def gb():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import deformetrica_code_gb300 as g
    return g


def mixture(rng, n, d):
    means = rng.uniform(0.15, 0.85, (8, d))
    return np.ascontiguousarray(np.clip(means[rng.integers(0, 8, n)] + 0.05 * rng.standard_normal((n, d)), 0, 1))


def test_synthetic_tuning_round_trips(gb, port, tmp_path):
    rng = np.random.default_rng(1)
    n, d, sigma = 20000, 3, 0.1
    X, Y, W, A = rng.random((n, d)), rng.random((n, d)), rng.standard_normal((n, d)), rng.standard_normal((n, d))
    ctx = gb.Context()
    ctx.autotune("convolve_gradient_alpha_fused", d, d, n, n, sigma)
    k = gb.GB300ExactKernel(d, sigma, context=ctx)
    k.SetSources(Y)
    k.SetWeights(W)
    v, g_ = k.ConvolveAndGradient(X, A)
    variant, nsplit = ctx.last_launch()
    assert variant in TWO_FLOAT_FAMILY and 1 <= nsplit <= n // 64
    assert normwise_rel(v, port.convolve(X, Y, W, sigma)) <= 2e-6
    assert normwise_rel(g_, port.grad_alpha(X, Y, W, sigma, A)) <= 2e-6
    path = str(tmp_path / "tune.jsonl")
    ctx.tune_save(path)
    lines = open(path).read().splitlines()
    assert len(lines) == 1 and '"path": 1' in lines[0]
    ctx2 = gb.Context()
    ctx2.tune_load(path)
    k2 = gb.GB300ExactKernel(d, sigma, context=ctx2)
    k2.SetSources(Y)
    k2.SetWeights(W)
    v2, g2 = k2.ConvolveAndGradient(X, A)
    assert ctx2.last_launch() == (variant, nsplit)
    assert np.array_equal(v, v2) and np.array_equal(g_, g2)
    os.environ["GBK_TUNE_FILE"] = path
    try:
        ctx3 = gb.Context()
    finally:
        del os.environ["GBK_TUNE_FILE"]
    k3 = gb.GB300ExactKernel(d, sigma, context=ctx3)
    k3.SetSources(Y)
    k3.SetWeights(W)
    assert np.array_equal(k3.ConvolveAndGradient(X, A)[0], v)
    assert ctx3.last_launch() == (variant, nsplit)


def test_data_tuning_on_the_spatial_path(gb, port):
    import torch
    rng = np.random.default_rng(2)
    n, d, sigma = 70000, 3, 0.05  # n^2 >= 2^30: the automatic order sorts
    x, y = mixture(rng, n, d), mixture(rng, n, d)
    w, a = rng.standard_normal((n, d)), rng.standard_normal((n, d))
    X, Y, W, A = (torch.from_numpy(t).cuda() for t in (x, y, w, a))
    ctx = gb.Context()
    k = gb.GB300ExactKernel(d, sigma, context=ctx)
    k.SetSources(Y)
    k.SetWeights(W)

    def timed():
        k.ConvolveAndGradient(X, A)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best = 1e30
        for _ in range(3):
            e0.record()
            out = k.ConvolveAndGradient(X, A)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best, out

    t_default, _ = timed()
    default_launch = ctx.last_launch()
    assert default_launch[0] == 11  # bulk staging is the spatial path's default
    variant, nsplit, ms = ctx.autotune_data("convolve_gradient_alpha_fused", X, Y, W, sigma, alpha=A)
    assert variant in SPATIAL_FAMILY and nsplit >= 1 and ms > 0
    t_tuned, (v, g_) = timed()
    assert ctx.last_launch() == (variant, nsplit)
    print("default", default_launch, f"{t_default:.3f} ms; tuned", (variant, nsplit), f"{t_tuned:.3f} ms")
    assert t_tuned <= 1.05 * t_default
    it = np.sort(rng.choice(n, 1500, replace=False))
    xs, as_ = np.ascontiguousarray(x[it]), np.ascontiguousarray(a[it])
    assert normwise_rel(v.cpu().numpy()[it], port.convolve(xs, y, w, sigma)) <= 2e-6
    assert normwise_rel(g_.cpu().numpy()[it], port.grad_alpha(xs, y, w, sigma, as_)) <= 2e-6


def test_an_entry_from_another_family_is_ignored(gb, tmp_path):
    """A table line naming a one-float shape for the two-float path: the call keeps two-float."""
    rng = np.random.default_rng(3)
    n, d = 12000, 3
    path = str(tmp_path / "t.jsonl")
    bucket = int(np.log2(n))
    with open(path, "w") as f:
        f.write('{"op": 1, "mode": 0, "d": 3, "dv": 3, "bx": %d, "by": %d, "path": 1, "variant": 0, "nsplit": 2}\n'
                % (bucket, bucket))
    ctx = gb.Context()
    ctx.tune_load(path)
    k = gb.GB300ExactKernel(d, 0.1, context=ctx)
    k.SetSources(rng.random((n, d)))
    k.SetWeights(rng.standard_normal((n, d)))
    k.ConvolveAndGradient(rng.random((n, d)), rng.standard_normal((n, d)))
    assert ctx.last_launch()[0] in TWO_FLOAT_FAMILY


def test_untunable_requests_fail_cleanly(gb):
    ctx = gb.Context()
    with pytest.raises(gb.GBKError):
        ctx.autotune("special_hessian", 3, 3, 1000, 1000, 0.1)
    with pytest.raises(gb.GBKError):
        ctx.autotune("convolve", 3, 5, 1000, 1000, 0.1)  # dv 5 is not a compiled column width
