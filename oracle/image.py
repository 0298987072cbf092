"""FP64 numpy restatement of the reference's image-grid kernel path (TEST INFRASTRUCTURE ONLY: the
oracle of gbk_convolve_image_fast, gbk_convolve_gradient_image_fast(_alpha) and gbk_flow_image_maps).
The reference's code needs ITK images; ITK is not available here, so the index rounding and region
cropping are restated from ITK's documented behaviour. The three ExactKernel methods are pinned
against the reference's own compiled code run through ITK stand-ins with that behaviour
(oracle/ref_shim/, tests/golden/image_fast.npz); the reference has no test of this path.

* image points (GridFunctions::ImageToPoints, src/support/utilities/GridFunctions.cxx:41-60): one
  row per pixel in ITK iteration order (first index fastest), the physical point origin +
  spacing x index (identity direction);
* ExactKernel::ConvolveImageFast (src/support/kernels/ExactKernel.cxx:76-129): for each control
  point y_j in order, the region of 6 sigma pixels per axis (ITK Size::Fill of 6 sigma: truncated)
  starting at the index of the physical point y_j - 3 sigma (TransformPhysicalPointToIndex:
  rounded half up), cropped to the image (ImageRegion::Crop); every pixel p of it gets
  V[p] += W[j] K(X[p], y_j), K = exp(-|X[p] - y_j|^2 / sigma^2), X the rows of the (deformed) image
  points. A region that misses the image cannot be cropped and the reference's ITK region iterator
  throws: here a ValueError;
* ExactKernel::ConvolveGradientImageFast(X, image) (ExactKernel.cxx:207-257): the same windows; every
  pixel p of control point j's region gets G[p][k][l] += g_l W[j][k] with g = (X[p] - y_j) (-2 K / sigma^2)
  (EvaluateKernelGradient, ExactKernel.h:98-110); and ConvolveGradientImageFast(X, alpha, image)
  (:277-290): out[p][l] = sum_k G[p][k][l] alpha[p][k];
* Diffeos image maps (src/core/model_tools/deformations/Diffeos.cxx:725-770, the non-regression
  branch): maps[t] = image points for all t; if |mom[0]|_F < 1e-20 nothing moves; else backward
  from t = T-1: dY = conv(maps[t]; pos[t], mom[t]), maps[t-1] = maps[t] - dt dY, with Heun
  dY2 = conv(maps[t-1]; pos[t-1], mom[t-1]), maps[t-1] = maps[t] - (dY + dY2)(dt 0.5); after each
  step the bounding-box check (CheckBoundingBox, :187-198) stops the integration when a column of
  maps[t-1] leaves [bbox[k, 0], bbox[k, 1]].
"""
from __future__ import annotations

import numpy as np


def image_points(origin, spacing, size):
    """The pixels' physical points, first index fastest (ImageToPoints)."""
    origin, spacing = np.asarray(origin, float), np.asarray(spacing, float)
    d = len(size)
    idx = np.indices(tuple(size[::-1])).reshape(d, -1)[::-1].T  # rows: (i0, i1[, i2]), i0 fastest
    return origin + spacing * idx


def windows(y, sigma, origin, spacing, size):
    """(start, L, lo, hi, ok): each control point's region start index (rounded half up), the
    region size int(6 sigma), the cropped bounds [lo, hi) and whether the region meets the image."""
    origin, spacing = np.asarray(origin, float), np.asarray(spacing, float)
    size = np.asarray(size, np.int64)
    L = int(6 * sigma)
    start = np.floor((np.asarray(y, float) - 3 * sigma - origin) / spacing + 0.5).astype(np.int64)
    ok = np.all((start < size) & (start + L > 0), axis=1) & (L > 0)
    lo, hi = np.maximum(start, 0), np.minimum(start + L, size)
    return start, L, lo, hi, ok


def convolve_image_fast(x, y, w, sigma, origin, spacing, size):
    """ExactKernel::ConvolveImageFast: x (prod(size) x d) the image's (deformed) points, y, w the
    control points and momenta (ny x d)."""
    x, y, w = np.asarray(x, float), np.asarray(y, float), np.asarray(w, float)
    size = [int(s) for s in size]
    d = len(size)
    if x.shape[0] != int(np.prod(size)):
        raise ValueError("one row of x per pixel")
    if y.shape[0] != w.shape[0]:
        raise ValueError("Sources and weights count mismatch")
    _, _, lo, hi, ok = windows(y, sigma, origin, spacing, size)
    if not ok.all():
        raise ValueError(f"control point {int(np.argmin(ok))}: its region misses the image")
    strides = np.cumprod([1] + size[:-1])
    s2 = sigma * sigma
    V = np.zeros((x.shape[0], d))
    for j in range(y.shape[0]):
        axes = [np.arange(lo[j, k], hi[j, k]) for k in range(d)]
        grid = np.meshgrid(*axes, indexing="ij")
        rows = sum(g.ravel() * strides[k] for k, g in enumerate(grid))
        sq = np.zeros(rows.shape[0])
        for k in range(d):
            diff = x[rows, k] - y[j, k]
            sq += diff * diff
        K = np.exp(-sq / s2)
        V[rows] += w[j, :d] * K[:, None]
    return V


def convolve_gradient_image_fast(x, y, w, sigma, origin, spacing, size, alpha=None):
    """ExactKernel::ConvolveGradientImageFast: (prod(size) x dv x d) gradients, or with `alpha`
    (prod(size) x dv) their contraction (prod(size) x d)."""
    x, y, w = np.asarray(x, float), np.asarray(y, float), np.asarray(w, float)
    size = [int(s) for s in size]
    d = len(size)
    if x.shape[0] != int(np.prod(size)):
        raise ValueError("one row of x per pixel")
    if y.shape[0] != w.shape[0]:
        raise ValueError("Sources and weights count mismatch")
    _, _, lo, hi, ok = windows(y, sigma, origin, spacing, size)
    if not ok.all():
        raise ValueError(f"control point {int(np.argmin(ok))}: its region misses the image")
    strides = np.cumprod([1] + size[:-1])
    s2 = sigma * sigma
    G = np.zeros((x.shape[0], w.shape[1], d))
    for j in range(y.shape[0]):
        axes = [np.arange(lo[j, k], hi[j, k]) for k in range(d)]
        grid = np.meshgrid(*axes, indexing="ij")
        rows = sum(g.ravel() * strides[k] for k, g in enumerate(grid))
        diff = x[rows] - y[j]
        sq = np.zeros(rows.shape[0])
        for k in range(d):
            sq += diff[:, k] * diff[:, k]
        f = (-2.0 * np.exp(-sq / s2)) / s2
        g = diff * f[:, None]
        G[rows] += w[j][None, :, None] * g[:, None, :]
    if alpha is None:
        return G
    alpha = np.asarray(alpha, float)
    out = np.zeros((x.shape[0], d))
    for k in range(w.shape[1]):  # sum over k in order, as the reference's G^T alpha
        out += G[:, k, :] * alpha[:, k:k + 1]
    return out


def _exact_convolve(x, y, w, sigma):
    sq = ((x[:, None, :] - y[None, :, :]) ** 2).sum(-1)
    return np.exp(-sq / (sigma * sigma)) @ w


def flow_image_maps(pos, mom, sigma, origin, spacing, size, heun=True, fast=True, bbox=None, span=1.0):
    """Diffeos' backward integration of the image maps: (maps T x npix x d, stopped_at or None)."""
    pos, mom = np.asarray(pos, float), np.asarray(mom, float)
    T = pos.shape[0]
    pts = image_points(origin, spacing, size)
    maps = np.repeat(pts[None], T, axis=0)
    if np.linalg.norm(mom[0]) < 1e-20:
        return maps, None
    dt = span / (T - 1)

    def conv(X, t):
        if fast:
            return convolve_image_fast(X, pos[t], mom[t], sigma, origin, spacing, size)
        return _exact_convolve(X, pos[t], mom[t], sigma)

    for t in range(T - 1, 0, -1):
        dY = conv(maps[t], t)
        maps[t - 1] = maps[t] - dY * dt
        if heun:
            dY2 = conv(maps[t - 1], t - 1)
            maps[t - 1] = maps[t] - (dY + dY2) * (dt * 0.5)
        if bbox is not None:
            b = np.asarray(bbox, float)
            if np.any(maps[t - 1].min(axis=0) < b[:, 0]) or np.any(maps[t - 1].max(axis=0) > b[:, 1]):
                return maps, t - 1
    return maps, None
