"""Sums of term magnitudes for every kernel-sum output (dense numpy, small cases only).

For an output element s = sum_j t_j the FP32 path's error is bounded by ~u * sum_j |t_j|, not by
u * |s|: when the terms cancel (N(0,1) weights, the special Hessian's xi_j - xi_i) the plain
relative error says nothing about the arithmetic. The condition-aware error of an element is
|err| / sum_j |t_j|; these helpers give the denominator for each method of ExactKernel.

With ``exp_cond=True`` the sums describe the FP32 path's error model:
  * every term is weighted by (1 + a_ij + 2 sqrt(a_ij) R / (16 sigma)), a_ij = |x_i - y_j|^2 /
    sigma^2: the relative condition number of K = exp(-a) with respect to a is a, and rounding
    the centred coordinates to FP32 moves a by ~2 sqrt(a) u R / sigma;
  * every |x_i - y_j|_l factor becomes |x_i - y_j|_l + R / 16, because the rounded centred
    coordinates carry an ABSOLUTE error ~u R (u = 2^-24, R = the largest distance of a point from
    the targets' bounding-box centre) however small the difference itself is.
With the 1e-6 (~16 u) tolerance the R/16 slack stands for that u R. Rows whose every neighbour is
several sigma away, or whose dominant pair is aligned on an axis, are bounded by these sums.
"""
from __future__ import annotations

import numpy as np


EXP_COND = False
RADIUS = 0.0


def _dk(X, Y, sigma):
    D = X[:, None, :] - Y[None, :, :]
    a = np.sum(D * D, axis=2) / (sigma * sigma)
    K = np.exp(-a)
    if EXP_COND:
        K = K * (1.0 + a + 2.0 * np.sqrt(a) * RADIUS / (16.0 * sigma))
        D = np.abs(D) + RADIUS / 16.0
    return D, K


def radius(X, Y):
    """Largest |p - c|_inf over targets and sources, c = midpoint of the targets' bounding box."""
    c = 0.5 * (X.min(axis=0) + X.max(axis=0))
    return float(max(np.abs(X - c).max(), np.abs(Y - c).max()))


def convolve(X, Y, W, sigma):
    _, K = _dk(X, Y, sigma)
    return K @ np.abs(W)


def grad_varlin(X, Y, W, sigma):
    D, K = _dk(X, Y, sigma)
    return (2 / sigma**2) * np.einsum("ij,jk,ijl->ikl", K, np.abs(W), np.abs(D))


def grad_alpha(X, Y, W, sigma, A):
    D, K = _dk(X, Y, sigma)
    ab = np.abs(A) @ np.abs(W).T
    return (2 / sigma**2) * np.einsum("ij,ij,ijl->il", K, ab, np.abs(D))


def grad_dim(X, Y, W, sigma, dim):
    D, K = _dk(X, Y, sigma)
    return (2 / sigma**2) * (K * np.abs(D[:, :, dim])) @ np.abs(W)


def hess_full(X, Y, W, sigma):
    D, K = _dk(X, Y, sigma)
    d = X.shape[1]
    s2 = sigma * sigma
    H = 4 * np.abs(D[:, :, :, None] * D[:, :, None, :]) / s2**2 + (2 / s2) * np.eye(d)[None, None]
    return np.einsum("ij,jk,ijab->ikab", K, np.abs(W), H)


def hess_rowcol(X, Y, W, sigma, r, c):
    return hess_full(X, Y, W, sigma)[:, :, r, c]


def special_hessian(Y, B, sigma, XI):
    D, K = _dk(Y, Y, sigma)
    s2 = sigma * sigma
    bb = np.abs(B @ B.T)
    dxi = XI[None, :, :] - XI[:, None, :]  # xi_j - xi_i
    q = np.abs(np.sum(D * dxi, axis=2))
    return np.einsum("ij,ijl->il", bb * K, 4 / s2**2 * q[:, :, None] * np.abs(D) + 2 / s2 * np.abs(dxi))


def special_hessian_reference_noise(Y, B, sigma, XI):
    """Scale of the reference's own FP64 rounding noise in ConvolveSpecialHessian: it forms
    -sum_j bb H_ij xi_i and sum_j bb H_ij xi_j in separate sweeps (AbstractKernel.cxx:33-83), so
    even the j = i terms, which cancel exactly, leave ~1e-16 of sum_j |bb| |H_ij| (|xi_i| + |xi_j|)."""
    D, K = _dk(Y, Y, sigma)
    s2 = sigma * sigma
    bb = np.abs(B @ B.T)
    ax = np.abs(XI)
    amp = ax[:, None, :] + ax[None, :, :]
    H = 4 / s2**2 * np.abs(D)[:, :, :, None] * np.abs(D)[:, :, None, :] + 2 / s2 * np.eye(Y.shape[1])
    return np.einsum("ij,ijab,ijb->ia", bb * K, H, amp)


def condition_error(approx, ref, mag, floor=None):
    """max over elements of (|approx - ref| - floor)+ / mag (elements with mag == 0 must match
    exactly). `floor` is the absolute noise of the reference value itself, if any."""
    approx, ref, mag = (np.asarray(a, dtype=np.float64) for a in (approx, ref, mag))
    err = np.abs(approx - ref)
    if floor is not None:
        err = np.maximum(err - np.asarray(floor, dtype=np.float64), 0.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        r = np.where(mag > 0, err / mag, np.where(err > 0, np.inf, 0.0))
    return float(r.max()) if r.size else 0.0


def for_key(key, X, Y, W, sigma, A, W3, exp_cond=False):
    """Magnitude sums for the result named `key` in the golden fixtures."""
    global EXP_COND, RADIUS
    EXP_COND = exp_cond
    RADIUS = radius(X, Y) if exp_cond else 0.0
    try:
        return _for_key(key, X, Y, W, sigma, A, W3)
    finally:
        EXP_COND = False
        RADIUS = 0.0


def _for_key(key, X, Y, W, sigma, A, W3):
    d = X.shape[1]
    if key == "convolve":
        return convolve(X, Y, W, sigma)
    if key == "grad_varlin":
        return grad_varlin(X, Y, W, sigma)
    if key == "grad_alpha":
        return grad_alpha(X, Y, W, sigma, A)
    if key.startswith("grad_dim_x_"):
        return grad_dim(X, Y, W, sigma, int(key[-1]))
    if key.startswith("grad_dim_"):
        return grad_dim(Y, Y, W, sigma, int(key[-1]))
    if key == "grad_kdp":
        return grad_dim(X[:Y.shape[0]], Y, W[:, -1:], sigma, d - 1)[:, 0]
    if key == "hess_full":
        return hess_full(X, Y, W, sigma)
    if key.startswith("hess_rowcol_"):
        return hess_rowcol(X, Y, W, sigma, int(key[-2]), int(key[-1]))
    if key == "hess_kdpdq":
        return hess_full(X, Y, W[:, :1], sigma)[:, 0, 0, d - 1]
    if key == "special_hessian":
        global RADIUS
        if EXP_COND:
            RADIUS = radius(Y, Y)
        return special_hessian(Y, W3, sigma, W3)
    raise KeyError(key)
