"""Failure paths on the GPU without a GPU fault: an allocation failure injected on the host
(gbk_set_alloc_limit), empty inputs, and shape errors, each returning a status the caller reads
while the context stays usable. The reference throws std::runtime_error on shape mismatches
(ExactKernel.cxx:58-59) and returns empty or zero sums for empty inputs (its loops run zero times)."""
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


def test_injected_allocation_failure_leaves_the_context_usable(gb, K):
    rng = np.random.default_rng(1)
    x, y, w = rng.random((5000, 3)), rng.random((6000, 3)), rng.normal(size=(6000, 3))
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    ctx.set_alloc_limit(4096)  # host arrays are staged through device buffers larger than this
    k = gb.GB300ExactKernel(3, 0.2, context=ctx)
    k.SetSources(y)
    k.SetWeights(w)
    with pytest.raises(gb.GBKError) as e:
        k.Convolve(x)
    assert e.value.code == 4  # GBK_ERR_ALLOC
    assert "injected" in str(e.value)
    ctx.set_alloc_limit(0)
    v = k.Convolve(x)
    ref = K.convolve(x, y, w, 0.2)
    assert np.linalg.norm(v - ref) <= 1e-10 * np.linalg.norm(ref)
    ctx.set_alloc_limit(1 << 20)  # the P3M scratch is refused too
    with pytest.raises(gb.GBKError, match="injected"):
        gb.p3m_convolve(x, y, w, 0.2, context=ctx)
    ctx.set_alloc_limit(0)
    assert gb.p3m_convolve(x, y, w, 0.2, context=ctx).shape == (5000, 3)


def test_empty_inputs(gb):
    ctx = gb.Context()
    k = gb.GB300ExactKernel(3, 0.3, context=ctx)
    rng = np.random.default_rng(2)
    y, w = rng.random((40, 3)), rng.normal(size=(40, 3))
    k.SetSources(y)
    k.SetWeights(w)
    assert k.Convolve(np.zeros((0, 3))).shape == (0, 3)
    assert k.ConvolveGradient(np.zeros((0, 3)), np.zeros((0, 3))).shape == (0, 3)
    k.SetSources(np.zeros((0, 3)))
    k.SetWeights(np.zeros((0, 3)))
    x = rng.random((25, 3))
    assert np.array_equal(k.Convolve(x), np.zeros((25, 3)))
    assert np.array_equal(k.ConvolveGradient(x, rng.normal(size=(25, 3))), np.zeros((25, 3)))


def test_shape_errors_raise_and_the_context_survives(gb, K):
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    k = gb.GB300ExactKernel(3, 0.3, context=ctx)
    rng = np.random.default_rng(3)
    x, y, w = rng.random((30, 3)), rng.random((20, 3)), rng.normal(size=(20, 3))
    k.SetSources(y)
    k.SetWeights(w[:10])
    with pytest.raises(RuntimeError, match="count mismatch"):
        k.Convolve(x)
    k.SetWeights(w)
    with pytest.raises((ValueError, RuntimeError, gb.GBKError)):
        k.ConvolveGradient(x, np.zeros((7, 3)))
    v = k.Convolve(x)
    ref = K.convolve(x, y, w, 0.3)
    assert np.linalg.norm(v - ref) <= 1e-12 * np.linalg.norm(ref)
