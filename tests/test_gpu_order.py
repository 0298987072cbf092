"""GPU: spatial order of targets and sources (GBK_ORDER_* in include/gbk.h) against the FP64 oracle.

* Pruning is exact: SPATIAL (source chunks beyond the zero-kernel distance skipped) and
  SPATIAL_NOPRUNE (same order, every pair evaluated) give the same bits for every kernel-sum
  method in both precision modes, on clustered points with a small kernel width.
* The order changes nothing but the rounding: every method matches the oracle with outputs in
  caller row order, with and without source splits, for ragged and degenerate inputs.
* At small kernel widths the spatial order makes the compensated-FP32 path more accurate than
  caller order (each CTA's centred coordinates are smaller).
* AUTO orders large calls only.
Points follow the sweep workload: a mixture of 8 Gaussians (std 0.05, means uniform in
[0.15, 0.85]^d) clipped to [0, 1]^d, weights N(0, 1).
"""
import numpy as np
import pytest

from tests.conftest import normwise_rel, reference_compare

pytestmark = pytest.mark.gpu

F64_TOL = 1e-10
F32_NORM_TOL = 2e-6


@pytest.fixture(scope="module")
def gb():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import deformetrica_code_gb300 as g
    return g


@pytest.fixture(scope="module")
def ctx(gb):
    c = gb.Context()
    yield c
    c.set_order(gb.GBK_ORDER_AUTO)
    c.set_split(0)


def mixture(rng, n, d):
    means = rng.uniform(0.15, 0.85, (8, d))
    pts = means[rng.integers(0, 8, n)] + 0.05 * rng.standard_normal((n, d))
    return np.ascontiguousarray(np.clip(pts, 0.0, 1.0))


def kern(gb, ctx, d, sigma, Y, W, mode, order):
    ctx.set_mode(mode)
    ctx.set_order(order)
    k = gb.GB300ExactKernel(d, sigma, context=ctx)
    k.SetSources(Y)
    k.SetWeights(W)
    return k


def all_methods(k, X, A, Xi):
    d = X.shape[1]
    out = {"convolve": k.Convolve(X), "grad_alpha": k.ConvolveGradient(X, A), "grad_varlin": k.ConvolveGradient(X),
           "hess_full": k.ConvolveHessian(X), "hess_rowcol": k.ConvolveHessian(X, 0, d - 1)}
    for dim in range(d):
        out[f"grad_dim_{dim}"] = k.ConvolveGradient(X, dim)
    for q, v in enumerate(k.ForwardAdjoint(X, A)):
        out[f"fwd_adjoint_{q}"] = v
    out["special_hessian"] = k.ConvolveSpecialHessian(Xi)
    return out


@pytest.mark.parametrize("d", [2, 3])
def test_pruning_is_bit_exact(gb, ctx, d):
    rng = np.random.default_rng(31 + d)
    X, Y = mixture(rng, 6000, d), mixture(rng, 9000, d)
    W, A, Xi = rng.standard_normal((9000, d)), rng.standard_normal((6000, d)), rng.standard_normal((9000, d))
    for mode in (gb.GBK_MODE_F32C, gb.GBK_MODE_F64):
        got = {}
        for order in (gb.GBK_ORDER_SPATIAL, gb.GBK_ORDER_SPATIAL_NOPRUNE):
            k = kern(gb, ctx, d, 0.02, Y, W, mode, order)
            got[order] = all_methods(k, X, A, Xi)
        for key, v in got[gb.GBK_ORDER_SPATIAL].items():
            assert np.array_equal(v, got[gb.GBK_ORDER_SPATIAL_NOPRUNE][key]), (mode, key)
            assert np.isfinite(v).all()


@pytest.mark.parametrize("sigma", [0.02, 0.1, 0.5])
def test_spatial_order_matches_oracle(gb, ctx, port, sigma):
    rng = np.random.default_rng(int(sigma * 1000))
    d = 3
    X, Y = mixture(rng, 3000, d), mixture(rng, 5000, d)
    W, A = rng.standard_normal((5000, d)), rng.standard_normal((3000, d))
    ref = {"convolve": port.convolve(X, Y, W, sigma), "grad_alpha": port.grad_alpha(X, Y, W, sigma, A),
           "grad_varlin": port.grad_varlin(X, Y, W, sigma), "grad_dim_1": port.grad_dim(X, Y, W, sigma, 1),
           "hess_rowcol": port.hess_rowcol(X, Y, W, sigma, 0, 2)}
    for split in (1, 4, 0):
        ctx.set_split(split)
        for mode in (gb.GBK_MODE_F64, gb.GBK_MODE_F32C):
            k = kern(gb, ctx, d, sigma, Y, W, mode, gb.GBK_ORDER_SPATIAL)
            got = {"convolve": k.Convolve(X), "grad_alpha": k.ConvolveGradient(X, A),
                   "grad_varlin": k.ConvolveGradient(X), "grad_dim_1": k.ConvolveGradient(X, 1),
                   "hess_rowcol": k.ConvolveHessian(X, 0, 2)}
            for key, r in ref.items():
                if mode == gb.GBK_MODE_F64:
                    assert reference_compare(r, got[key], 1) <= F64_TOL, (split, key)
                else:
                    assert normwise_rel(got[key], r) <= F32_NORM_TOL, (split, key, normwise_rel(got[key], r))
    ctx.set_split(0)


def test_special_hessian_and_fwd_adjoint_spatial(gb, ctx, port):
    rng = np.random.default_rng(5)
    d, sigma = 3, 0.05
    Y, X = mixture(rng, 4000, d), mixture(rng, 2500, d)
    W, Xi, A = rng.standard_normal((4000, d)), rng.standard_normal((4000, d)), rng.standard_normal((2500, d))
    r_sh = port.special_hessian(Y, W, sigma, Xi)
    r_fa = port.fwd_adjoint(X, Y, W, sigma, A)
    for mode, tol in ((gb.GBK_MODE_F64, 1e-12), (gb.GBK_MODE_F32C, F32_NORM_TOL)):
        k = kern(gb, ctx, d, sigma, Y, W, mode, gb.GBK_ORDER_SPATIAL)
        e_sh = normwise_rel(k.ConvolveSpecialHessian(Xi), r_sh)
        for g_, r_ in zip(k.ForwardAdjoint(X, A), r_fa):
            assert normwise_rel(g_, r_) <= tol
        # the special Hessian cancels xi_j - xi_i: hold the spatial order to the caller order's error
        k_off = kern(gb, ctx, d, sigma, Y, W, mode, gb.GBK_ORDER_OFF)
        e_off = normwise_rel(k_off.ConvolveSpecialHessian(Xi), r_sh)
        assert e_sh <= max(2 * e_off, tol), (mode, e_sh, e_off)


def test_small_sigma_accuracy_improves(gb, ctx, port):
    """sigma = 0.02 on the mixture: caller order leaves CTAs whose targets span the whole set."""
    rng = np.random.default_rng(3)
    d, sigma, n = 3, 0.02, 20000
    X, Y = mixture(rng, n, d), mixture(rng, n, d)
    W, A = rng.standard_normal((n, d)), rng.standard_normal((n, d))
    rv, rg = port.convolve(X, Y, W, sigma), port.grad_alpha(X, Y, W, sigma, A)
    err = {}
    for order in (gb.GBK_ORDER_OFF, gb.GBK_ORDER_SPATIAL):
        k = kern(gb, ctx, d, sigma, Y, W, gb.GBK_MODE_F32C, order)
        v, g = k.ConvolveAndGradient(X, A)
        err[order] = (normwise_rel(v, rv), normwise_rel(g, rg))
    print("normwise error (convolve, gradient): caller order", err[gb.GBK_ORDER_OFF], "spatial",
          err[gb.GBK_ORDER_SPATIAL])
    assert err[gb.GBK_ORDER_SPATIAL][0] <= 1e-6 and err[gb.GBK_ORDER_SPATIAL][1] <= 1e-6
    assert err[gb.GBK_ORDER_SPATIAL][0] < err[gb.GBK_ORDER_OFF][0]
    assert err[gb.GBK_ORDER_SPATIAL][1] < err[gb.GBK_ORDER_OFF][1]


@pytest.mark.parametrize("nx,ny,d", [(1, 1, 3), (7, 300, 3), (513, 1, 3), (1025, 777, 2), (4096, 4096, 2)])
def test_ragged_and_degenerate(gb, ctx, port, nx, ny, d):
    rng = np.random.default_rng(nx + 17 * ny)
    X, Y = mixture(rng, nx, d), mixture(rng, ny, d)
    W, A = rng.standard_normal((ny, d)), rng.standard_normal((nx, d))
    for sigma in (0.01, 0.3):
        rv, rg = port.convolve(X, Y, W, sigma), port.grad_alpha(X, Y, W, sigma, A)
        for mode in (gb.GBK_MODE_F64, gb.GBK_MODE_F32C):
            k = kern(gb, ctx, d, sigma, Y, W, mode, gb.GBK_ORDER_SPATIAL)
            v, g = k.ConvolveAndGradient(X, A)
            if mode == gb.GBK_MODE_F64:
                assert reference_compare(rv, v, 1) <= F64_TOL and reference_compare(rg, g, 1) <= F64_TOL
            else:
                assert normwise_rel(v, rv) <= F32_NORM_TOL and normwise_rel(g, rg) <= F32_NORM_TOL


def test_identical_points(gb, ctx, port):
    """All targets and all sources at one point: a zero-extent box, one cell."""
    X = np.full((1500, 3), 0.25)
    Y = np.full((2000, 3), 0.25)
    rng = np.random.default_rng(2)
    W = rng.standard_normal((2000, 3))
    rv = port.convolve(X, Y, W, 0.1)
    for mode in (gb.GBK_MODE_F64, gb.GBK_MODE_F32C):
        k = kern(gb, ctx, 3, 0.1, Y, W, mode, gb.GBK_ORDER_SPATIAL)
        assert normwise_rel(k.Convolve(X), rv) <= 1e-6


def test_device_pointers_same_bits(gb, ctx):
    import torch
    rng = np.random.default_rng(4)
    X, Y = mixture(rng, 5000, 3), mixture(rng, 7000, 3)
    W = rng.standard_normal((7000, 3))
    k = kern(gb, ctx, 3, 0.03, Y, W, gb.GBK_MODE_F32C, gb.GBK_ORDER_SPATIAL)
    vh = k.Convolve(X)
    dev = lambda a: torch.from_numpy(a).cuda()
    k2 = kern(gb, ctx, 3, 0.03, dev(Y), dev(W), gb.GBK_MODE_F32C, gb.GBK_ORDER_SPATIAL)
    vd = k2.Convolve(dev(X)).cpu().numpy()
    torch.cuda.synchronize()
    assert np.array_equal(vh, vd)


def test_evaluated_pair_count(gb, ctx):
    """Caller order and SPATIAL_NOPRUNE evaluate every pair; SPATIAL skips pairs at small sigma only."""
    rng = np.random.default_rng(8)
    X, Y = mixture(rng, 5000, 3), mixture(rng, 7000, 3)
    W = rng.standard_normal((7000, 3))

    def pairs(order, sigma):
        k = kern(gb, ctx, 3, sigma, Y, W, gb.GBK_MODE_F32C, order)
        p0 = ctx.evaluated_pairs()
        k.Convolve(X)
        return ctx.evaluated_pairs() - p0

    assert pairs(gb.GBK_ORDER_OFF, 0.02) == 5000 * 7000
    assert pairs(gb.GBK_ORDER_SPATIAL_NOPRUNE, 0.02) == 5000 * 7000
    assert pairs(gb.GBK_ORDER_SPATIAL, 3.0) == 5000 * 7000
    assert pairs(gb.GBK_ORDER_SPATIAL, 0.02) < 0.6 * 5000 * 7000


def test_auto_orders_large_calls_only(gb, ctx):
    rng = np.random.default_rng(6)

    def launches(order, n):
        k = kern(gb, ctx, 3, 0.1, rng.random((n, 3)), rng.standard_normal((n, 3)), gb.GBK_MODE_F32C, order)
        x = rng.random((n, 3))
        n0 = ctx.launch_count()
        k.Convolve(x)
        return ctx.launch_count() - n0

    # the order adds, per point set, a box and a keys kernel and (up to 16384 points) a one-CTA sort
    # (the device radix sort above that is counted as the library's), then one tiles kernel for the
    # targets and one kernel for the source boxes and copies; pruning adds the targets' non-finite
    # scan and the conditional unbounding of the chunk boxes
    assert launches(gb.GBK_ORDER_AUTO, 12000) == launches(gb.GBK_ORDER_OFF, 12000)
    assert launches(gb.GBK_ORDER_AUTO, 40000) == launches(gb.GBK_ORDER_OFF, 40000) + 8
    assert launches(gb.GBK_ORDER_SPATIAL, 1000) == launches(gb.GBK_ORDER_OFF, 1000) + 10
    assert launches(gb.GBK_ORDER_SPATIAL, 20000) == launches(gb.GBK_ORDER_OFF, 20000) + 8

    # forward + adjoint: x and y are sorted once each for both passes
    def fa_launches(order, n):
        k = kern(gb, ctx, 3, 0.1, rng.random((n, 3)), rng.standard_normal((n, 3)), gb.GBK_MODE_F32C, order)
        x, al = rng.random((n, 3)), rng.standard_normal((n, 3))
        n0 = ctx.launch_count()
        k.ForwardAdjoint(x, al)
        return ctx.launch_count() - n0

    assert fa_launches(gb.GBK_ORDER_SPATIAL, 1000) == fa_launches(gb.GBK_ORDER_OFF, 1000) + 14
    with pytest.raises(gb.GBKError):
        ctx.set_order(7)
