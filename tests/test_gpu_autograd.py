"""GPU: the torch.autograd wrapper over the C ABI (deformetrica_code_gb300/autograd.py).

* torch.autograd.gradcheck in the FP64 mode: the hand-written adjoint (gbk_forward_adjoint) against
  central finite differences of the forward kernel sum, for X, Y and W together, d = 2 and 3.
* The adjoint's dL/dX against ExactKernel::ConvolveGradient(X, alpha) (the oracle, pinned to the
  compiled reference) with alpha = dL/dV, and dL/dW, dL/dY against their kernel-sum definitions,
  in both precision modes.
"""
import numpy as np
import pytest

from tests.conftest import normwise_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import deformetrica_code_gb300 as g
    return g


@pytest.mark.parametrize("d", [2, 3])
def test_gradcheck_fp64(gb, d):
    import torch
    from deformetrica_code_gb300.autograd import gaussian_convolve
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    g = torch.Generator().manual_seed(11 + d)
    X = torch.rand(7, d, dtype=torch.float64, generator=g).cuda().requires_grad_()
    Y = torch.rand(9, d, dtype=torch.float64, generator=g).cuda().requires_grad_()
    W = torch.randn(9, d, dtype=torch.float64, generator=g).cuda().requires_grad_()
    f = lambda x, y, w: gaussian_convolve(x, y, w, 0.4, ctx)
    assert torch.autograd.gradcheck(f, (X, Y, W), eps=1e-6, atol=1e-8, rtol=1e-6)


@pytest.mark.parametrize("mode_name,tol", [("f64", 1e-11), ("f32c", 2e-6)])
def test_backward_matches_oracle(gb, port, mode_name, tol):
    import torch
    from deformetrica_code_gb300.autograd import gaussian_convolve
    mode = gb.GBK_MODE_F64 if mode_name == "f64" else gb.GBK_MODE_F32C
    ctx = gb.Context(mode=mode)
    rng = np.random.default_rng(21)
    x, y = rng.random((600, 3)), rng.random((800, 3))
    w, gv = rng.standard_normal((800, 3)), rng.standard_normal((600, 3))
    X, Y, W = (torch.from_numpy(a).cuda().requires_grad_() for a in (x, y, w))
    V = gaussian_convolve(X, Y, W, 0.2, ctx)
    V.backward(torch.from_numpy(gv).cuda())
    assert normwise_rel(V.detach().cpu().numpy(), port.convolve(x, y, w, 0.2)) <= tol
    # dL/dX = ConvolveGradient(X, alpha = dL/dV) with sources Y, weights W
    assert normwise_rel(X.grad.cpu().numpy(), port.grad_alpha(x, y, w, 0.2, gv)) <= tol
    # dL/dW = K(Y, X) dL/dV and dL/dY = ConvolveGradient(Y, W) with sources X, weights dL/dV
    assert normwise_rel(W.grad.cpu().numpy(), port.convolve(y, x, gv, 0.2)) <= tol
    assert normwise_rel(Y.grad.cpu().numpy(), port.grad_alpha(y, x, gv, 0.2, w)) <= tol
