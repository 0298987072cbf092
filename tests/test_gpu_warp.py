"""GPU: the warp-split kernels (gbk_pairs_warp.cuh: VARIANT_WARP, VARIANT_WARP_TWO_FLOAT), which run
kernel sums too small for the default launch shape in caller order -- 64 targets per CTA shared by 8
warps that divide the sources, coordinates packed once per launch -- against the FP64 oracle.

* Convolve, the alpha-gradient and the fused forward + adjoint over ragged sizes (targets not a
  multiple of 64, sources not a multiple of the 256 a CTA's warps stage per round, fewer sources
  than warps x 32, a single source), every compiled weight width, d = 2 and 3, one-float and
  adaptive two-float coordinates, with and without cross-CTA source splits;
* repeated launches are bitwise equal (fixed warp and split order);
* the fused control-point adjoint update (OpAdjointCP) through ComputeUpdateAt;
* the launch takes the warp-split variant (gbk_last_launch).
"""
import numpy as np
import pytest

from tests.conftest import normwise_rel

pytestmark = pytest.mark.gpu

VARIANT_WARP, VARIANT_WARP_TWO_FLOAT = 13, 14
# normwise against FP64 (one-float coordinates on narrow data, two-float ones on wide data)
TOL = {"off": 1e-6, "two_float": 1e-6}


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


def mixture(rng, n, means):
    d = means.shape[1]
    return np.ascontiguousarray(means[rng.integers(0, len(means), n)] + 0.05 * rng.standard_normal((n, d)))


@pytest.mark.parametrize("d", [2, 3])
@pytest.mark.parametrize("order", ["off", "two_float"])
def test_warp_split_matches_oracle_on_ragged_sizes(gb, ctx, port, d, order):
    rng = np.random.default_rng(70 + d)
    ctx.set_order(gb.GBK_ORDER_OFF if order == "off" else gb.GBK_ORDER_TWO_FLOAT)
    want = VARIANT_WARP if order == "off" else VARIANT_WARP_TWO_FLOAT
    dvs = (1, 2, 3, 4) if d == 2 else (1, 2, 3, 6)
    for nx, ny in ((1000, 1000), (97, 1001), (333, 257), (64, 31), (5, 1), (1000, 10242)):
        # clusters shared by targets and sources: within ~8 scaled units for one-float coordinates,
        # over ~22 (2.8 / 0.15 x 1.2) for two-float ones, so that wide CTAs occur
        means = rng.uniform(0.15, 0.85, (8, d)) if order == "off" else rng.uniform(0.6, 3.4, (8, d))
        X, Y = mixture(rng, nx, means), mixture(rng, ny, means)
        if ny < 32:  # a few sources: next to targets, so that no output is only far-away terms
            Y = np.ascontiguousarray(X[rng.integers(0, nx, ny)] + 0.02 * rng.standard_normal((ny, d)))
        sigma = 0.15
        for dv in dvs:
            W, A = rng.standard_normal((ny, dv)), rng.standard_normal((nx, dv))
            k = gb.GB300ExactKernel(d, sigma, context=ctx)
            k.SetSources(Y)
            k.SetWeights(W)
            for split in (0, 2, 5):
                ctx.set_split(split)
                v = k.Convolve(X)
                assert ctx.last_launch()[0] == want, (nx, ny, dv, ctx.last_launch())
                assert normwise_rel(v, port.convolve(X, Y, W, sigma)) <= TOL[order], (nx, ny, dv, split)
                ga = k.ConvolveGradient(X, A)
                assert normwise_rel(ga, port.grad_alpha(X, Y, W, sigma, A)) <= TOL[order], (nx, ny, dv, split)
                assert np.array_equal(k.Convolve(X), v)  # bitwise reproducible
            ctx.set_split(0)
            if dv == d:
                got = k.ForwardAdjoint(X, A)
                for g_, r_ in zip(got, port.fwd_adjoint(X, Y, W, sigma, A)):
                    assert normwise_rel(g_, r_) <= TOL[order], (nx, ny, dv)
    ctx.set_order(gb.GBK_ORDER_AUTO)


def test_warp_split_adjoint_update_matches_seven_calls(gb, ctx, port):
    """ComputeUpdateAt's fused control-point pass on the warp-split kernel (caller order, FP32C)
    against the reference's five control-point calls and two landmark calls."""
    from oracle import deformation as D
    from deformetrica_code_gb300.deformation import Deformation
    rng = np.random.default_rng(12)
    ctx.set_mode(gb.GBK_MODE_F32C)
    for d in (2, 3):
        for ncp in (57, 1000):
            cp = rng.uniform(0.2, 0.8, (ncp, d))
            mom, xp, xm = (rng.standard_normal((ncp, d)) for _ in range(3))
            lm, th = rng.uniform(0.1, 0.9, (911, d)), rng.standard_normal((911, d))
            ref = D.compute_update_at(port, 0.15, cp, mom, xp, xm, lm, th)
            df = Deformation(d, 0.15, 2, context=ctx)
            got = df.compute_update_at(cp, mom, xp, xm, lm, th)
            for g_, r_ in zip(got, ref):
                assert normwise_rel(g_, r_) <= 2e-6, (d, ncp)
            again = df.compute_update_at(cp, mom, xp, xm, lm, th)
            for g_, a_ in zip(got, again):
                assert np.array_equal(g_, a_)
