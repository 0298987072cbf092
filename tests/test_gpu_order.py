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


@pytest.mark.parametrize("d", [2, 3])
def test_two_float_coordinates(gb, ctx, port, d):
    """GBK_ORDER_TWO_FLOAT: caller order with hi + lo coordinates for Convolve and the alpha-gradient
    in every CTA whose targets spread wider than 16 scaled units. On the mixture at sigma = 0.02
    (spread ~60 units) it is more accurate than one-float caller order, with and without source splits
    and in the small launch shape; at sigma = 0.5 (spread ~2.4 units) every CTA runs the one-float
    loop and gives the caller order's bits, as do ops without a two-float variant and the FP64 mode."""
    rng = np.random.default_rng(40 + d)
    sigma = 0.02
    for nx, ny in ((6000, 9000), (700, 500)):  # the default shape; the small shape
        X, Y = mixture(rng, nx, d), mixture(rng, ny, d)
        W, A = rng.standard_normal((ny, d)), rng.standard_normal((nx, d))
        ref = port.fwd_adjoint(X, Y, W, sigma, A)
        err = {}
        for order in (gb.GBK_ORDER_OFF, gb.GBK_ORDER_TWO_FLOAT):
            for split in (0, 3):
                ctx.set_split(split)
                k = kern(gb, ctx, d, sigma, Y, W, gb.GBK_MODE_F32C, order)
                got = k.ForwardAdjoint(X, A)
                v = k.Convolve(X)
                assert np.array_equal(v, got[0])  # Convolve alone = the fused pass's first output
                err[order, split] = max(normwise_rel(g_, r_) for g_, r_ in zip(got, ref))
        ctx.set_split(0)
        print(d, nx, ny, "worst normwise: caller order", err[gb.GBK_ORDER_OFF, 0], "two-float",
              err[gb.GBK_ORDER_TWO_FLOAT, 0])
        for split in (0, 3):
            assert err[gb.GBK_ORDER_TWO_FLOAT, split] <= 5e-7
            assert err[gb.GBK_ORDER_TWO_FLOAT, split] < err[gb.GBK_ORDER_OFF, split]
    X, Y = mixture(rng, 3000, d), mixture(rng, 4000, d)
    W, A = rng.standard_normal((4000, d)), rng.standard_normal((3000, d))
    for nx in (3000, 300):  # the default and the small shape
        same = [kern(gb, ctx, d, 0.5, Y, W, gb.GBK_MODE_F32C, order).ForwardAdjoint(X[:nx], A[:nx])
                for order in (gb.GBK_ORDER_OFF, gb.GBK_ORDER_TWO_FLOAT)]
        for a_, b_ in zip(*same):
            assert np.array_equal(a_, b_)
    for mode in (gb.GBK_MODE_F32C, gb.GBK_MODE_F64):
        outs = {}
        for order in (gb.GBK_ORDER_OFF, gb.GBK_ORDER_TWO_FLOAT):
            k = kern(gb, ctx, d, sigma, Y, W, mode, order)
            outs[order] = (k.ConvolveGradient(X), k.ConvolveHessian(X, 0, 1)) + \
                ((k.Convolve(X),) if mode == gb.GBK_MODE_F64 else ())
        for a_, b_ in zip(outs[gb.GBK_ORDER_OFF], outs[gb.GBK_ORDER_TWO_FLOAT]):
            assert np.array_equal(a_, b_)
    ctx.set_mode(gb.GBK_MODE_F32C)


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
    # scan and the conditional unbounding of the chunk boxes. Below 2^30 pairs AUTO runs Convolve
    # and the alpha-gradient in caller order (adaptive two-float variant: same launches as OFF). The
    # small shape packs the coordinates once per launch in caller order (one launch), not in the
    # spatial order.
    assert launches(gb.GBK_ORDER_AUTO, 1000) == launches(gb.GBK_ORDER_OFF, 1000) == 2
    assert launches(gb.GBK_ORDER_AUTO, 12000) == launches(gb.GBK_ORDER_OFF, 12000)
    assert launches(gb.GBK_ORDER_AUTO, 40000) == launches(gb.GBK_ORDER_OFF, 40000) + 8
    assert launches(gb.GBK_ORDER_SPATIAL, 1000) == launches(gb.GBK_ORDER_OFF, 1000) + 10 - 1
    assert launches(gb.GBK_ORDER_SPATIAL, 20000) == launches(gb.GBK_ORDER_OFF, 20000) + 8

    # other ops from 2^22 pairs measure the extent of the two point sets first (one box launch):
    # uniform points in [0, 1]^3 span 12 units of the FP32 coordinate scale at sigma 0.1 (caller
    # order) and 60 at sigma 0.02 (the spatial order)
    def launches_at(order, n, sigma, op="convolve"):
        k = kern(gb, ctx, 3, sigma, rng.random((n, 3)), rng.standard_normal((n, 3)), gb.GBK_MODE_F32C, order)
        x = rng.random((n, 3))
        n0 = ctx.launch_count()
        if op == "convolve":
            k.Convolve(x)
        else:
            k.ConvolveGradient(x)  # varlin: no two-float variant
        return ctx.launch_count() - n0

    assert launches_at(gb.GBK_ORDER_AUTO, 20000, 0.02) == launches_at(gb.GBK_ORDER_OFF, 20000, 0.02)
    assert launches_at(gb.GBK_ORDER_AUTO, 12000, 0.02, "varlin") == \
        launches_at(gb.GBK_ORDER_SPATIAL, 12000, 0.02, "varlin") + 1
    assert launches_at(gb.GBK_ORDER_AUTO, 12000, 0.1, "varlin") == launches_at(gb.GBK_ORDER_OFF, 12000, 0.1, "varlin") + 1
    assert launches_at(gb.GBK_ORDER_AUTO, 1000, 0.02, "varlin") == launches_at(gb.GBK_ORDER_OFF, 1000, 0.02, "varlin")

    # forward + adjoint: x and y are sorted once each for both passes
    def fa_launches(order, n):
        k = kern(gb, ctx, 3, 0.1, rng.random((n, 3)), rng.standard_normal((n, 3)), gb.GBK_MODE_F32C, order)
        x, al = rng.random((n, 3)), rng.standard_normal((n, 3))
        n0 = ctx.launch_count()
        k.ForwardAdjoint(x, al)
        return ctx.launch_count() - n0

    # (caller order packs the coordinates for each of the two small-shape passes)
    assert fa_launches(gb.GBK_ORDER_SPATIAL, 1000) == fa_launches(gb.GBK_ORDER_OFF, 1000) + 14 - 2
    assert fa_launches(gb.GBK_ORDER_AUTO, 12000) == fa_launches(gb.GBK_ORDER_OFF, 12000)
    with pytest.raises(gb.GBKError):
        ctx.set_order(7)


@pytest.mark.parametrize("d", [2, 3])
@pytest.mark.parametrize("n", [10000, 30000])
def test_default_order_meets_1e6_on_the_sweep_grid(gb, port, n, d):
    """The large kernel-sum sweep's workload (8-Gaussian mixture, seed 3) at its two smallest sizes and
    every kernel width, in the library's default order (GBK_ORDER_AUTO, nothing forced): each of the
    four forward + adjoint outputs within 1e-6 of the FP64 oracle on 2048 sampled rows against all n
    partners, both normwise (max_i |err_i| / max_i |ref_i|) and condition-aware (per element,
    |err| / sum_j (1 + a_ij) |term_j| with a_ij = |x_i - y_j|^2 / sigma^2, the exponent's condition
    number). At sigma = 0.02 the points span ~60 units of the FP32 coordinate scale; caller order
    with one-float coordinates gave 1.2-1.4e-6 normwise there, so AUTO switches to two-float
    coordinates (n = 1e4) or the spatial order (n = 3e4). The plain-magnitude error (denominator
    sum_j |term_j|) is printed too: for a target whose nearest sources are several sigma away it is
    bounded below by ~2u a_ij in any FP32 evaluation, whatever the order."""
    import ctypes
    import torch
    import bench
    x, y, w, a = bench.make_workload(n, n, d=d, seed=3)
    X, Y, W, A = (torch.from_numpy(t).cuda() for t in (x, y, w, a))
    outs = [torch.empty_like(X) for _ in range(4)]
    c = gb.Context()
    c.use_torch_stream()
    assert c.get_order() == gb.GBK_ORDER_AUTO
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    rng = np.random.default_rng(7)
    it = np.sort(rng.choice(n, size=2048, replace=False))
    jt = np.sort(rng.choice(n, size=2048, replace=False))
    xs, ys, as_, ws = (np.ascontiguousarray(t) for t in (x[it], y[jt], a[it], w[jt]))
    report = []
    for sigma in (0.02, 0.1, 0.5):
        c.check(c.lib.gbk_forward_adjoint(c.h, d, d, p(X), n, p(Y), p(W), n, sigma, p(A), *[p(o) for o in outs]))
        torch.cuda.synchronize()
        v, gx, gy, gw = (o.cpu().numpy() for o in outs)
        cases = {"v": (v[it], port.convolve(xs, y, w, sigma), lambda cd: port.convolve_mag(xs, y, w, sigma, cd)),
                 "gx": (gx[it], port.grad_alpha(xs, y, w, sigma, as_),
                        lambda cd: port.grad_alpha_mag(xs, y, w, sigma, as_, cd)),
                 "gy": (gy[jt], port.grad_alpha(ys, x, a, sigma, ws),
                        lambda cd: port.grad_alpha_mag(ys, x, a, sigma, ws, cd)),
                 "gw": (gw[jt], port.convolve(ys, x, a, sigma), lambda cd: port.convolve_mag(ys, x, a, sigma, cd))}
        for key, (got, r, mag) in cases.items():
            e = np.abs(got - r)
            nw = float(np.linalg.norm(got - r, axis=1).max() / np.linalg.norm(r, axis=1).max())
            cond = float((e / np.maximum(mag(True), 1e-300)).max())
            plain = float((e / np.maximum(mag(False), 1e-300)).max())
            report.append((sigma, key, nw, cond, plain, float(e.max())))
    print("\n".join(f"d={d} n={n} sigma={s_} {k}: normwise {nw:.2e} condition-aware {cd:.2e} "
                    f"plain-magnitude {pl:.2e} max abs {ma:.2e}" for s_, k, nw, cd, pl, ma in report))
    for s_, k, nw, cd, _, _ in report:
        assert nw <= 1e-6 and cd <= 1e-6, (s_, k, nw, cd)


@pytest.mark.parametrize("d,dv", [(3, 3), (2, 2), (3, 6)])
def test_bulk_staging_is_bit_exact(gb, ctx, d, dv):
    """GBK_STAGING_BULK (cp.async.bulk into a double-buffered shared area, mbarrier completion)
    stages the same source records as ordinary loads: the spatial order's results are bitwise equal,
    pruned and unpruned, with and without source splits, for a source count that is not a multiple of
    the chunk; the launch reports the bulk variant, and no bounded wait gives up."""
    rng = np.random.default_rng(70 + d + dv)
    nx, ny = 20000, 30001  # enough work for the default launch shape (the small one has no bulk variant)
    X, Y = mixture(rng, nx, d), mixture(rng, ny, d)
    W, A = rng.standard_normal((ny, dv)), rng.standard_normal((nx, dv))
    for order in (gb.GBK_ORDER_SPATIAL, gb.GBK_ORDER_SPATIAL_NOPRUNE):
        for split in (0, 3):
            ctx.set_split(split)
            got = {}
            for staging in (gb.GBK_STAGING_LOADS, gb.GBK_STAGING_BULK):
                ctx.set_staging(staging)
                k = kern(gb, ctx, d, 0.03, Y, W, gb.GBK_MODE_F32C, order)
                got[staging] = (k.Convolve(X),) + k.ConvolveAndGradient(X, A) + k.ForwardAdjoint(X, A)
                variant, _ = ctx.last_launch()
                assert (variant == 11) == (staging == gb.GBK_STAGING_BULK)
                ctx.synchronize()
            for a_, b_ in zip(got[gb.GBK_STAGING_LOADS], got[gb.GBK_STAGING_BULK]):
                assert np.array_equal(a_, b_)
    ctx.set_split(0)
    ctx.set_staging(gb.GBK_STAGING_AUTO)


def test_bulk_staging_128_thread_shape(gb, tmp_path):
    """The bulk-staged 128-thread shape (12, a tuner choice) against the load-staged one (4) with the
    same split count, set through a tuning table: the same bits."""
    import numpy as np
    rng = np.random.default_rng(81)
    nx, ny, d = 20000, 30001, 3
    X, Y = mixture(rng, nx, d), mixture(rng, ny, d)
    W, A = rng.standard_normal((ny, d)), rng.standard_normal((nx, d))
    b = lambda n: int(np.log2(n))
    got = {}
    for variant in (4, 12):
        path = str(tmp_path / f"t{variant}.jsonl")
        with open(path, "w") as f:
            f.write('{"op": 1, "mode": 0, "d": 3, "dv": 3, "bx": %d, "by": %d, "path": 2, "variant": %d, "nsplit": 3}\n'
                    % (b(nx), b(ny), variant))
        c = gb.Context()
        c.tune_load(path)
        k = kern(gb, c, d, 0.03, Y, W, gb.GBK_MODE_F32C, gb.GBK_ORDER_SPATIAL)
        got[variant] = k.ConvolveAndGradient(X, A)
        assert c.last_launch() == (variant, 3)
        c.synchronize()
    for a_, b_ in zip(got[4], got[12]):
        assert np.array_equal(a_, b_)


def test_bulk_staging_across_prune_windows(gb, ctx):
    """More than 4096 source chunks (two visit-mask windows) at a small width, where most chunks are
    pruned: the bulk path's look-ahead to the next visited chunk crosses the window boundary."""
    import torch
    rng = np.random.default_rng(77)
    X, Y = mixture(rng, 3000, 3), mixture(rng, 1_100_000, 3)
    W = rng.standard_normal((1_100_000, 3))
    dev = lambda a: torch.from_numpy(a).cuda()
    Xd, Yd, Wd = dev(X), dev(Y), dev(W)
    got = {}
    for staging in (gb.GBK_STAGING_LOADS, gb.GBK_STAGING_BULK):
        ctx.set_staging(staging)
        k = kern(gb, ctx, 3, 0.01, Yd, Wd, gb.GBK_MODE_F32C, gb.GBK_ORDER_SPATIAL)
        p0 = ctx.evaluated_pairs()
        got[staging] = k.Convolve(Xd).cpu().numpy()
        got[staging, "pairs"] = ctx.evaluated_pairs() - p0
        ctx.synchronize()
    assert np.array_equal(got[gb.GBK_STAGING_LOADS], got[gb.GBK_STAGING_BULK])
    assert got[gb.GBK_STAGING_LOADS, "pairs"] == got[gb.GBK_STAGING_BULK, "pairs"] < 0.5 * 3000 * 1_100_000
    ctx.set_staging(gb.GBK_STAGING_AUTO)


@pytest.mark.parametrize("d", [2, 3])
def test_small_shape_packed_coordinates_far_from_the_origin(gb, ctx, port, d):
    """Problems too small for the default launch shape run the small shape, which centres
    coordinates packed once per launch (hi + lo floats of the scaled coordinates) in FP32 with an
    exact TwoSum: accuracy must not depend on how far the points sit from the origin. Every output
    of the fused forward + adjoint and the ops without a fused form stay within FP32C tolerance of
    the FP64 oracle with the data moved 1e3 and 1e5 units away, in caller order and two-float."""
    rng = np.random.default_rng(90 + d)
    X0, Y0 = mixture(rng, 700, d), mixture(rng, 500, d)
    W, A = rng.standard_normal((500, d)), rng.standard_normal((700, d))
    sigma = 0.1
    for offset in (0.0, 1e3, 1e5):
        X, Y = X0 + offset, Y0 + offset
        ref = port.fwd_adjoint(X, Y, W, sigma, A)
        ref_varlin = port.grad_varlin(X, Y, W, sigma)
        for order in (gb.GBK_ORDER_OFF, gb.GBK_ORDER_TWO_FLOAT):
            k = kern(gb, ctx, d, sigma, Y, W, gb.GBK_MODE_F32C, order)
            got = k.ForwardAdjoint(X, A)
            for g_, r_ in zip(got, ref):
                assert normwise_rel(g_, r_) <= 5e-7, (offset, order)
            assert normwise_rel(np.asarray(k.ConvolveGradient(X)).reshape(ref_varlin.shape), ref_varlin) <= 5e-7
            assert ctx.last_launch()[0] == 8, ctx.last_launch()  # varlin ran the small shape (variant 8)
    ctx.set_order(gb.GBK_ORDER_AUTO)
