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


def test_memory_of_another_gpu_is_refused_before_any_launch(gb, K):
    """Device pointers that live on another GPU than the context's cannot be read by its kernels
    (no peer access is set up), so every entry point refuses them with GBK_ERR_ARG and queues
    nothing. With one GPU the other device is injected (gbk_inject_pointer_device)."""
    import ctypes
    import torch
    rng = np.random.default_rng(9)
    x, y, w = rng.random((300, 3)), rng.random((400, 3)), rng.normal(size=(400, 3))
    X, Y, W = (torch.from_numpy(t).cuda() for t in (x, y, w))
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    k = gb.GB300ExactKernel(3, 0.2, context=ctx)
    k.SetSources(Y)
    k.SetWeights(W)
    ctx.inject_pointer_device(ctx.device + 1)
    n0 = ctx.launch_count()
    with pytest.raises(gb.GBKError, match="another GPU") as e:
        k.Convolve(X)
    assert e.value.code == 1
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    assert ctx.lib.gbk_kernel_norm(ctx.h, 3, 3, p(Y), p(W), 400, 0.2, p(out)) == 1
    assert ctx.lib.gbk_kernel_norm_noalloc(ctx.h, 3, 3, p(Y), p(W), 400, 0.2, p(out)) == 1
    assert b"another GPU" in ctx.lib.gbk_last_error(ctx.h)
    assert ctx.launch_count() == n0
    # host arrays are staged, not read in place: unaffected
    kh = gb.GB300ExactKernel(3, 0.2, context=ctx)
    kh.SetSources(y)
    kh.SetWeights(w)
    ref = K.convolve(x, y, w, 0.2)
    assert np.linalg.norm(kh.Convolve(x) - ref) <= 1e-12 * np.linalg.norm(ref)
    ctx.inject_pointer_device(-1)
    v = k.Convolve(X).cpu().numpy()
    assert np.linalg.norm(v - ref) <= 1e-12 * np.linalg.norm(ref)


def _cudart():
    import ctypes
    import glob
    import os
    for d in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/sbsa-linux/lib",
              "/usr/local/cuda/targets/x86_64-linux/lib"):
        for f in sorted(glob.glob(os.path.join(d, "libcudart.so*"))):
            try:
                return ctypes.CDLL(f)
            except OSError:
                pass
    pytest.skip("libcudart not found")


def test_a_stream_already_in_error_returns_a_status(gb, K):
    """The caller hands the library a stream whose capture sequence is already invalidated (the
    caller synchronised it mid-capture): every operation queued on it fails. The call returns a
    GBK_ERR_* status with a message instead of crashing, and the context works again on its own
    stream. Nothing runs on the GPU while the stream is in error, so nothing can fault."""
    import ctypes
    import torch
    rt = _cudart()
    rng = np.random.default_rng(10)
    x, y, w = rng.random((700, 3)), rng.random((900, 3)), rng.normal(size=(900, 3))
    X, Y, W = (torch.from_numpy(t).cuda() for t in (x, y, w))
    V = torch.zeros_like(X)
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    ctx.check(ctx.lib.gbk_convolve(ctx.h, 3, 3, p(X), 700, p(Y), p(W), 900, 0.2, p(V)))  # buffers sized
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    h = ctypes.c_void_p(s.cuda_stream)
    assert rt.cudaStreamBeginCapture(h, 2) == 0  # cudaStreamCaptureModeRelaxed
    assert rt.cudaStreamSynchronize(h) != 0  # illegal while capturing: invalidates the capture
    ctx.check(ctx.lib.gbk_set_stream(ctx.h, h))
    rc = ctx.lib.gbk_convolve(ctx.h, 3, 3, p(X), 700, p(Y), p(W), 900, 0.2, p(V))
    assert rc in (3, 6), rc  # GBK_ERR_CUDA or GBK_ERR_STATE
    assert ctx.lib.gbk_last_error(ctx.h)
    graph = ctypes.c_void_p()
    assert rt.cudaStreamEndCapture(h, ctypes.byref(graph)) != 0  # the invalidated capture ends
    rt.cudaGetLastError()
    ctx.check(ctx.lib.gbk_set_stream(ctx.h, None))
    ctx.check(ctx.lib.gbk_convolve(ctx.h, 3, 3, p(X), 700, p(Y), p(W), 900, 0.2, p(V)))
    ctx.check(ctx.lib.gbk_synchronize(ctx.h))
    ref = K.convolve(x, y, w, 0.2)
    assert np.linalg.norm(V.cpu().numpy() - ref) <= 1e-12 * np.linalg.norm(ref)
