"""Non-finite inputs under the spatial order with exact-zero pruning: the reference's sums
(ExactKernel.cxx:51-74, 264-275) carry a NaN or an infinity into every target it meets, however
small the kernel value (0 x NaN = NaN, 0 x inf = NaN), so a chunk of sources holding one, or a
launch whose targets hold one, is never pruned. FP64 mode, where the kernel values underflow where
the reference's do: the NaN / inf pattern and the finite values match the FP64 oracle."""
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


@pytest.fixture(scope="module")
def K():
    import oracle
    return oracle.load("port")


def _case(seed=4, nx=6000, ny=9000):
    rng = np.random.default_rng(seed)
    x, y = 10 * rng.random((nx, 3)), 10 * rng.random((ny, 3))  # [0, 10]^3: exact zeros beyond 27 sigma
    w, a = rng.normal(size=(ny, 3)), rng.normal(size=(nx, 3))
    return x, y, w, a


def _same(got, ref):
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    assert np.array_equal(np.isposinf(got), np.isposinf(ref))
    assert np.array_equal(np.isneginf(got), np.isneginf(ref))
    fin = np.isfinite(ref)
    if fin.any():
        assert np.abs(got[fin] - ref[fin]).max() <= 1e-10 * np.abs(ref[fin]).max()


@pytest.mark.parametrize("where", ["source_weight_nan", "source_weight_inf", "source_point_nan",
                                   "target_point_nan", "target_alpha_nan"])
@pytest.mark.parametrize("order", ["SPATIAL", "OFF"])
def test_nonfinite_inputs_propagate_as_in_the_reference(gb, K, where, order):
    sigma = 0.1  # most source chunks are exact zeros for most target tiles
    x, y, w, a = _case()
    if where == "source_weight_nan":
        w[1234, 1] = np.nan
    elif where == "source_weight_inf":
        w[777, 0] = np.inf
    elif where == "source_point_nan":
        y[4321, 2] = np.nan
    elif where == "target_point_nan":
        x[55, 0] = np.nan
    else:
        a[99, 2] = np.nan
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    ctx.set_order(getattr(gb, f"GBK_ORDER_{order}"))
    k = gb.GB300ExactKernel(3, sigma, context=ctx)
    k.SetSources(y)
    k.SetWeights(w)
    v = k.Convolve(x)
    g = k.ConvolveGradient(x, a)
    _same(v, K.convolve(x, y, w, sigma))
    _same(g, K.grad_alpha(x, y, w, sigma, a))
    if where == "source_weight_nan":  # every target's column 1, however far from the source
        assert np.isnan(v[:, 1]).all() and np.isfinite(v[:, [0, 2]]).all()
    if where == "source_point_nan":
        assert np.isnan(v).all()
    if where == "target_point_nan":
        assert np.isnan(v[55]).all() and np.isfinite(np.delete(v, 55, axis=0)).all()
    if where == "source_weight_inf":  # 0 x inf where the kernel value is an exact zero
        assert np.isnan(v[:, 0]).any() and np.isinf(v[:, 0]).any()


def test_finite_inputs_still_pruned(gb):
    """The checks leave pruning on for finite inputs: fewer pairs are evaluated than N x M."""
    x, y, w, _ = _case(seed=7)
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    ctx.set_order(gb.GBK_ORDER_SPATIAL)
    k = gb.GB300ExactKernel(3, 0.1, context=ctx)
    k.SetSources(y)
    k.SetWeights(w)
    n0 = ctx.evaluated_pairs()
    k.Convolve(x)
    n1 = ctx.evaluated_pairs()
    assert 0 < n1 - n0 < 0.5 * x.shape[0] * y.shape[0]
    x[10, 1] = np.inf  # a non-finite target: the whole launch is evaluated
    k.Convolve(x)
    assert ctx.evaluated_pairs() - n1 == x.shape[0] * y.shape[0]
