"""gbk_kernel_norm_noalloc: the RKHS norm for callers that cannot allocate device memory.

Its scratch lives in a fixed __device__ array inside the library instead of context buffers grown
with cudaMalloc, for code that runs inside a memory budget fixed at start-up or from a pre-sized
pool. This file is collected last (tests/test_zz_*) so that a run stopping at the first failure
has run every other test first; it passes alone in a fresh process as well.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCRATCH_DOUBLES = 2 << 20


@pytest.fixture(scope="module")
def setup():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import deformetrica_code_gb300 as g
    return g, torch


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("mode,tol", [(0, 2e-6), (1, 1e-12)])
def test_noalloc_norm_matches_allocating_entry_point_twice(setup, mode, tol):
    g, torch = setup
    ctx = g.Context(mode=mode)
    ctx.use_torch_stream()
    lib = ctx.lib
    rng = np.random.default_rng(21)
    n, d, dv, sigma = 20000, 3, 3, 0.1
    Y = torch.from_numpy(rng.random((n, d))).cuda()
    W = torch.from_numpy(rng.standard_normal((n, dv))).cuda()
    ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    ctx.check(lib.gbk_kernel_norm(ctx.h, d, dv, _p(Y), _p(W), n, sigma, _p(ref)))
    outs = []
    for _ in range(2):  # two calls in a row share (and reuse) the scratch array
        out = torch.full((1,), np.nan, dtype=torch.float64, device="cuda")
        assert lib.gbk_kernel_norm_noalloc(ctx.h, d, dv, _p(Y), _p(W), n, sigma, _p(out)) == 0
        outs.append(out)
    torch.cuda.synchronize()
    r = float(ref.item())
    for out in outs:
        assert abs(float(out.item()) - r) <= tol * abs(r)


def test_noalloc_dv_chunks_and_d2(setup):
    g, torch = setup
    ctx = g.Context()
    ctx.use_torch_stream()
    rng = np.random.default_rng(5)
    n, d, dv = 3000, 2, 5  # dv = 5 runs as column chunks
    Y = torch.from_numpy(rng.random((n, d))).cuda()
    W = torch.from_numpy(rng.standard_normal((n, dv))).cuda()
    ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    ctx.check(ctx.lib.gbk_kernel_norm(ctx.h, d, dv, _p(Y), _p(W), n, 0.2, _p(ref)))
    for _ in range(2):
        assert ctx.lib.gbk_kernel_norm_noalloc(ctx.h, d, dv, _p(Y), _p(W), n, 0.2, _p(out)) == 0
        torch.cuda.synchronize()
        assert abs(out.item() - ref.item()) <= 2e-6 * abs(ref.item())


def test_noalloc_rejects_oversize_and_host_pointers(setup):
    g, torch = setup
    ctx = g.Context()
    lib = ctx.lib
    n = SCRATCH_DOUBLES // 3 + 1  # n * dv just above the scratch capacity
    Y = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    W = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert lib.gbk_kernel_norm_noalloc(ctx.h, 3, 3, _p(Y), _p(W), n, 0.1, _p(out)) == g._lib.GBK_ERR_ARG
    host = np.zeros((10, 3))
    assert lib.gbk_kernel_norm_noalloc(ctx.h, 3, 3, ctypes.c_void_p(host.ctypes.data), _p(W), 10, 0.1,
                                       _p(out)) == g._lib.GBK_ERR_ARG


def test_noalloc_allocates_nothing_and_counts_its_launches(setup):
    """The entry point's claim itself: after a first call (which may load the module holding the
    scratch array), further calls leave the device's free memory unchanged, and their launches are
    counted like every other entry point's."""
    g, torch = setup
    ctx = g.Context()
    ctx.use_torch_stream()
    lib = ctx.lib
    rng = np.random.default_rng(33)
    n, d, dv = 50000, 3, 3
    Y = torch.from_numpy(rng.random((n, d))).cuda()
    W = torch.from_numpy(rng.standard_normal((n, dv))).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert lib.gbk_kernel_norm_noalloc(ctx.h, d, dv, _p(Y), _p(W), n, 0.1, _p(out)) == 0
    torch.cuda.synchronize()
    first = float(out.item())
    free0, _ = torch.cuda.mem_get_info()
    n0 = ctx.launch_count()
    for _ in range(3):
        assert lib.gbk_kernel_norm_noalloc(ctx.h, d, dv, _p(Y), _p(W), n, 0.1, _p(out)) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert ctx.launch_count() - n0 >= 3 * 2  # pair kernel(s) + the FP64 dot, per call
    assert float(out.item()) == first  # bitwise reproducible, scratch reused


def test_noalloc_rejects_nan_width_with_a_message(setup):
    g, torch = setup
    ctx = g.Context()
    Y = torch.zeros((100, 3), dtype=torch.float64, device="cuda")
    W = torch.zeros((100, 3), dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    assert ctx.lib.gbk_kernel_norm_noalloc(ctx.h, 3, 3, _p(Y), _p(W), 100, float("nan"), _p(out)) == g._lib.GBK_ERR_ARG
    assert b"NaN" in ctx.lib.gbk_last_error(ctx.h)
