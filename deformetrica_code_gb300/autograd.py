"""torch.autograd.Function over the C ABI, used for gradcheck and finite-difference checks only.

Forward: V = Convolve(X) with sources Y and weights W (ExactKernel.cxx:51-74).
Backward: the library's hand-written adjoint (gbk_forward_adjoint) with alpha = dL/dV, which
returns dL/dX (= ConvolveGradient(X, alpha), ExactKernel.cxx:264-275), dL/dY and dL/dW from two
fused passes that recompute distances and exponentials instead of storing them.
"""
from __future__ import annotations

import ctypes

import torch

from ._lib import GBK_MODE_F64
from .kernel import Context, _ptr


class GaussianConvolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X, Y, W, sigma: float, kctx: Context):
        X, Y, W = X.contiguous(), Y.contiguous(), W.contiguous()
        d, dv = X.shape[1], W.shape[1]
        V = torch.empty((X.shape[0], dv), dtype=torch.float64, device=X.device)
        kctx.bind_stream(X, Y, W)
        kctx.check(kctx.lib.gbk_forward_adjoint(kctx.h, d, dv, _ptr(X), X.shape[0], _ptr(Y), _ptr(W),
                                                Y.shape[0], sigma, None, _ptr(V), None, None, None))
        ctx.save_for_backward(X, Y, W)
        ctx.sigma, ctx.kctx = sigma, kctx
        return V

    @staticmethod
    def backward(ctx, gV):
        X, Y, W = ctx.saved_tensors
        kctx, sigma = ctx.kctx, ctx.sigma
        gV = gV.contiguous()
        d, dv = X.shape[1], W.shape[1]
        gx = torch.empty_like(X)
        gy = torch.empty_like(Y)
        gw = torch.empty_like(W)
        kctx.bind_stream(X, Y, W, gV)
        kctx.check(kctx.lib.gbk_forward_adjoint(kctx.h, d, dv, _ptr(X), X.shape[0], _ptr(Y), _ptr(W),
                                                Y.shape[0], sigma, _ptr(gV), None, _ptr(gx), _ptr(gy),
                                                _ptr(gw)))
        return gx, gy, gw, None, None


def gaussian_convolve(X, Y, W, sigma: float, kctx: Context | None = None):
    """V_i = sum_j exp(-|X_i - Y_j|^2 / sigma^2) W_j with a differentiable (X, Y, W)."""
    return GaussianConvolve.apply(X, Y, W, float(sigma), kctx or Context(mode=GBK_MODE_F64))
