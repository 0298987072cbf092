"""FP64 numpy restatement of the reference's P3MKernel (TEST INFRASTRUCTURE ONLY: the oracle of the
library's GPU particle-mesh kernel). The reference's P3MKernel needs ITK with FFTW or VNL FFT
filters, which are not available here, so this restatement cannot be checked against the
reference's binary: parity with the reference's P3M is unpinned. Against the exact kernel it
carries the approximation error of the method (the reference's tests accept 8e-2).

The algorithm (src/support/kernels/P3MKernel.cxx):
* grid (DetermineGrids, :371-432): spacing = working-spacing-ratio x sigma in every dimension;
  per dimension the data-domain length plus 2 x padding-factor x sigma, divided by the spacing and
  truncated, rounded up to a power of two; the origin centres the grid on the domain;
* splatting (UpdateGrids, :237-347): each source's weights go to the 2^d grid points around it
  with multilinear weights (_getInterpolationWeightsAndGridPoints_2/_3, :473-593: only points
  inside the grid and weights > 0), skipping "border" points whose index is <= the grid padding
  (0) in any dimension;
* kernel images (BuildFFTKernel, :666-804; BuildFFTGradientKernels, :808-944): the Gaussian
  exp(-|x - c|^2 / sigma^2) and its gradient (x - c)(-2 K / sigma^2) at every non-border grid point,
  c the grid centre origin + size spacing / 2, moved by an inverse FFT shift so that c is at index 0;
* convolution (ApplyKernelFFT, :1088-1178): inverse FFT of FFT(splatted) x FFT(kernel), i.e. the
  circular convolution of the splatted weights with the kernel image;
* interpolation (Interpolate, :641-662): multilinear at the targets with the same weights.
Convolve (:1245-1355) interpolates the dv convolved grids; ConvolveGradient(X) (:1386-1447) the
d x dv gradient-kernel grids; ConvolveGradient(X, alpha) (:1357-1366) contracts it with alpha.
"""
from __future__ import annotations

import math

import numpy as np


def grid(lo, hi, sigma: float, ratio: float = 0.2, padding: float = 3.0):
    """(origin, size, spacing) of DetermineGrids: size a power of two per dimension."""
    s = ratio * sigma
    origin, size = [], []
    for l, h in zip(lo, hi):
        length = h - l
        n = int((length + 2 * padding * sigma) / s)
        l2 = math.log(float(n)) / math.log(2.0)
        t = int(l2)
        l2 = t + 1 if l2 - t > 0 else t
        n = int(2.0 ** l2)
        origin.append(l - (n * s - length) / 2)
        size.append(n)
    return np.array(origin), np.array(size, dtype=np.int64), s


def corners(p, origin, size, s):
    """The multilinear interpolation points and weights of one point (in the reference's corner
    order), points outside the grid and zero weights dropped."""
    d = len(p)
    c = (np.asarray(p, float) - origin) / s
    i1 = np.floor(c).astype(np.int64)
    f = c - i1
    g = (i1 + 1) - c
    out = []
    for bits in np.ndindex(*(2,) * d):  # first dimension slowest, as the reference's macro order
        ind = i1 + np.array(bits)
        w = 1.0
        for k in range(d):
            w *= f[k] if bits[k] else g[k]
        if np.all(ind >= 0) and np.all(ind < size) and w > 0:
            out.append((tuple(ind), w))
    return out


def upper_pairs(d):
    """The Hessian entries (r, c), r <= c, in the reference's order (BuildFFTHessianKernels)."""
    return [(r, c) for r in range(d) for c in range(r, d)]


def _kernel_images(origin, size, s, sigma, hessian=False):
    d = len(size)
    idx = np.indices(size)
    border = np.any(idx <= 0, axis=0)
    x = origin.reshape((d,) + (1,) * d) + idx * s
    c = origin + 0.5 * size * s
    diff = x - c.reshape((d,) + (1,) * d)
    s2 = sigma * sigma
    k = np.exp(-np.sum(diff * diff, axis=0) / s2)
    k[border] = 0.0
    grads = [np.where(border, 0.0, diff[p] * (-2.0 * k / s2)) for p in range(d)]
    shift = lambda a: np.fft.ifftshift(a)
    if not hessian:
        return shift(k), [shift(g) for g in grads]
    # ExactKernel::EvaluateKernelHessian (ExactKernel.h:113-132) at every non-border grid point
    hess = []
    for r, cc in upper_pairs(d):
        h = diff[r] * diff[cc] * (4.0 * k / (s2 * s2))
        if r == cc:
            h = h - 2.0 * k / s2
        hess.append(shift(np.where(border, 0.0, h)))
    return shift(k), [shift(g) for g in grads], hess


def _splat(y, w, origin, size, s):
    dv = w.shape[1]
    grids = np.zeros((dv,) + tuple(size))
    for i in range(len(y)):
        for ind, wt in corners(y[i], origin, size, s):
            if any(j <= 0 for j in ind):  # border points (grid padding 0) receive nothing
                continue
            grids[(slice(None),) + ind] += wt * w[i]
    return grids


def _interp(x, images, origin, size, s):
    out = np.zeros((len(x), len(images)))
    for i in range(len(x)):
        for ind, wt in corners(x[i], origin, size, s):
            for j, img in enumerate(images):
                out[i, j] += wt * img[ind]
    return out


def _conv(a, k):
    axes = tuple(range(a.ndim))
    return np.fft.irfftn(np.fft.rfftn(a, axes=axes) * np.fft.rfftn(k, axes=axes), s=a.shape, axes=axes)


def domain_of(x, y):
    both = np.concatenate([x, y])
    return both.min(axis=0), both.max(axis=0)


def convolve(x, y, w, sigma, lo=None, hi=None, ratio: float = 0.2, padding: float = 3.0):
    """P3MKernel::Convolve at targets x (nx x d) of sources y with weights w (ny x dv); the data
    domain [lo, hi] defaults to the bounding box of x and y."""
    if lo is None:
        lo, hi = domain_of(x, y)
    origin, size, s = grid(lo, hi, sigma, ratio, padding)
    k, _ = _kernel_images(origin, size, s, sigma)
    grids = _splat(y, np.asarray(w, float), origin, size, s)
    return _interp(x, [_conv(g, k) for g in grids], origin, size, s)


def convolve_gradient(x, y, w, sigma, lo=None, hi=None, ratio: float = 0.2, padding: float = 3.0):
    """P3MKernel::ConvolveGradient(X): (nx, dv, d), entry [i, k, p] from the gradient kernel p
    applied to weight column k."""
    if lo is None:
        lo, hi = domain_of(x, y)
    origin, size, s = grid(lo, hi, sigma, ratio, padding)
    _, gk = _kernel_images(origin, size, s, sigma)
    grids = _splat(y, np.asarray(w, float), origin, size, s)
    d, dv = len(size), grids.shape[0]
    images = [_conv(grids[k], gk[p]) for k in range(dv) for p in range(d)]
    return _interp(x, images, origin, size, s).reshape(len(x), dv, d)


def convolve_gradient_alpha(x, y, w, sigma, alpha, lo=None, hi=None, ratio: float = 0.2, padding: float = 3.0):
    """P3MKernel::ConvolveGradient(X, alpha) = G_i^T alpha_i."""
    g = convolve_gradient(x, y, w, sigma, lo, hi, ratio, padding)
    return np.einsum("ikp,ik->ip", g, np.asarray(alpha, float))


def convolve_gradient_dim(x, y, w, sigma, dim, lo=None, hi=None, ratio: float = 0.2, padding: float = 3.0):
    """P3MKernel::ConvolveGradient(X, dim) (:1443-1504): nx x dv, the gradient kernel `dim`."""
    if lo is None:
        lo, hi = domain_of(x, y)
    origin, size, s = grid(lo, hi, sigma, ratio, padding)
    _, gk = _kernel_images(origin, size, s, sigma)
    grids = _splat(y, np.asarray(w, float), origin, size, s)
    return _interp(x, [_conv(g, gk[dim]) for g in grids], origin, size, s)


def convolve_hessian(x, y, w, sigma, lo=None, hi=None, ratio: float = 0.2, padding: float = 3.0):
    """P3MKernel::ConvolveHessian(X) (:1549-1620): (nx, dv, d, d), symmetric."""
    if lo is None:
        lo, hi = domain_of(x, y)
    origin, size, s = grid(lo, hi, sigma, ratio, padding)
    _, _, hk = _kernel_images(origin, size, s, sigma, hessian=True)
    grids = _splat(y, np.asarray(w, float), origin, size, s)
    d, dv, pairs = len(size), grids.shape[0], upper_pairs(len(size))
    vals = _interp(x, [_conv(grids[k], hk[p]) for p in range(len(pairs)) for k in range(dv)], origin, size, s)
    out = np.zeros((len(x), dv, d, d))
    for p, (r, c) in enumerate(pairs):
        for k in range(dv):
            out[:, k, r, c] = out[:, k, c, r] = vals[:, k + dv * p]
    return out


def convolve_hessian_rowcol(x, y, w, sigma, row, col, lo=None, hi=None, ratio: float = 0.2, padding: float = 3.0):
    """P3MKernel::ConvolveHessian(X, row, col) (:1622-1687): nx x dv."""
    if lo is None:
        lo, hi = domain_of(x, y)
    origin, size, s = grid(lo, hi, sigma, ratio, padding)
    _, _, hk = _kernel_images(origin, size, s, sigma, hessian=True)
    grids = _splat(y, np.asarray(w, float), origin, size, s)
    p = upper_pairs(len(size)).index((min(row, col), max(row, col)))
    return _interp(x, [_conv(g, hk[p]) for g in grids], origin, size, s)


def special_hessian(y, w, sigma, xi, lo=None, hi=None, ratio: float = 0.2, padding: float = 3.0):
    """AbstractKernel::ConvolveSpecialHessian (AbstractKernel.cxx:22-88) composed from this P3M's
    ConvolveHessian(Y) and ConvolveHessian(Y, r, q) with the reference's re-weightings (P3MKernel
    inherits it): N x d for sources y, weights beta = w (N x d) and xi (N x d)."""
    y, beta, xi = (np.asarray(a, float) for a in (y, w, xi))
    if lo is None:
        lo, hi = domain_of(y, y)
    n, d = y.shape
    ha = convolve_hessian(y, y, beta, sigma, lo, hi, ratio, padding)  # (N, dv = d, d, d)
    out = np.zeros((n, d))
    for i in range(n):
        aux = np.zeros((d, d))
        for dim in range(d):
            aux -= ha[i, dim] * beta[i, dim]
        out[i] = aux @ xi[i]
    H = np.zeros((n, d, d))
    for r in range(d):
        wd = beta * xi[:, r:r + 1]
        hrr = convolve_hessian_rowcol(y, y, wd, sigma, r, r, lo, hi, ratio, padding)
        H[:, r, :] += hrr
        for q in range(r + 1, d):
            wt = np.concatenate([wd, beta * xi[:, q:q + 1]], axis=1)
            hrq = convolve_hessian_rowcol(y, y, wt, sigma, r, q, lo, hi, ratio, padding)
            H[:, q, :] += hrq[:, :d]
            H[:, r, :] += hrq[:, d:]
    return out + np.einsum("irc,ic->ir", H, beta)
