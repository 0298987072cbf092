"""FP64 restatement of the reference's surface and curve data terms (TEST INFRASTRUCTURE ONLY).

Surface currents: OrientedSurfaceMesh.cxx:124-352. Surface varifolds: NonOrientedSurfaceMesh.cxx:
124-378. Curve currents: OrientedPolyLine.cxx (ComputeMatch, ComputeMatchGradient,
UpdateCentersTangents, UpdateSelfNorm). Curve varifolds: NonOrientedPolyLine.cxx:125-300, 364-378. Point clouds:
PointCloud.cxx:104-254. Volume meshes: OrientedVolumeMesh.cxx:115-367. Landmarks:
Landmark.cxx:288-322. Every kernel sum goes through the kernel oracle, as the reference goes through its kernel object.
Meshes are (points nv x d, cells nf x 3 or nf x 2 int) arrays; the reference reads them from VTK.
"""
from __future__ import annotations

import numpy as np

from .kernels import OracleLib


def centers_normals(pts, tris):
    """OrientedSurfaceMesh::UpdateCentersNormals, :298-328: c = mean of the vertices,
    n = (p2 - p0) x (p1 - p0) / 2."""
    p0, p1, p2 = pts[tris[:, 0]], pts[tris[:, 1]], pts[tris[:, 2]]
    return (p0 + p1 + p2) / 3.0, np.cross(p2 - p0, p1 - p0) / 2


def currents_norm(K: OracleLib, sigma, c, n):
    """UpdateSelfNorm, :330-352: sum_f n_f . (K n)_f."""
    return float(np.sum(K.convolve(c, c, n, sigma) * n))


def currents_match(K: OracleLib, sigma, pts_s, tris_s, pts_t, tris_t):
    """ComputeMatch, :124-163: |T|^2 + |S|^2 - 2 <S, T>."""
    cs, ns = centers_normals(pts_s, tris_s)
    ct, nt = centers_normals(pts_t, tris_t)
    m = currents_norm(K, sigma, ct, nt) + currents_norm(K, sigma, cs, ns)
    sdt = K.convolve(ct, cs, ns, sigma)
    return m - 2.0 * float(np.sum(sdt * nt))


def currents_match_gradient(K: OracleLib, sigma, pts_s, tris_s, pts_t, tris_t):
    """ComputeMatchGradient, :165-241: gradient with respect to the vertices of S."""
    cs, ns = centers_normals(pts_s, tris_s)
    ct, nt = centers_normals(pts_t, tris_t)
    ktau_s = K.convolve(cs, cs, ns, sigma)
    gk_s = K.grad_alpha(cs, cs, ns, sigma, ns)
    ktau_t = K.convolve(cs, ct, nt, sigma)
    gk_t = K.grad_alpha(cs, ct, nt, sigma, ns)
    gktau = (gk_s - gk_t) * 2.0 / 3.0
    grad = np.zeros_like(pts_s)
    p = pts_s
    i0, i1, i2 = tris_s[:, 0], tris_s[:, 1], tris_s[:, 2]
    e0, e1, e2 = p[i2] - p[i1], p[i0] - p[i2], p[i1] - p[i0]
    kt = ktau_s - ktau_t
    for idx, e in ((i0, e0), (i1, e1), (i2, e2)):
        np.add.at(grad, idx, np.cross(e, kt) + gktau)
    return grad


def varifold_normals(pts, tris):
    """NonOrientedSurfaceMesh::UpdateCentersNormals, :269-310: n / sqrt(|n| + 1e-20) and the
    upper-triangle products n_p n_q (p <= q)."""
    c, n = centers_normals(pts, tris)
    n = n / np.sqrt(np.linalg.norm(n, axis=1) + 1e-20)[:, None]
    iu = np.triu_indices(3)
    mn = (n[:, :, None] * n[:, None, :])[:, iu[0], iu[1]]
    return c, n, mn


def special_product(M, X):
    """NonOrientedSurfaceMesh::special_product, :364-378 (NonOrientedPolyLine::special_product for
    any d): the symmetric d x d matrix of the d(d+1)/2 upper-triangle entries M times X."""
    d = X.shape[-1]
    iu = np.triu_indices(d)
    S = np.zeros(M.shape[:-1] + (d, d))
    S[..., iu[0], iu[1]] = M
    S[..., iu[1], iu[0]] = M
    return np.einsum("...pq,...q->...p", S, X)


def varifold_norm(K: OracleLib, sigma, c, n, mn):
    kw = K.convolve(c, c, mn, sigma)
    return float(np.sum(n * special_product(kw, n)))


def varifold_match(K: OracleLib, sigma, pts_s, tris_s, pts_t, tris_t):
    """NonOrientedSurfaceMesh::ComputeMatch, :124-165."""
    cs, ns, ms = varifold_normals(pts_s, tris_s)
    ct, nt, mt = varifold_normals(pts_t, tris_t)
    m = varifold_norm(K, sigma, ct, nt, mt) + varifold_norm(K, sigma, cs, ns, ms)
    sdt = K.convolve(ct, cs, ms, sigma)
    return m - 2.0 * float(np.sum(nt * special_product(sdt, nt)))


def varifold_match_gradient(K: OracleLib, sigma, pts_s, tris_s, pts_t, tris_t):
    """NonOrientedSurfaceMesh::ComputeMatchGradient, :169-265."""
    cs, ns, ms = varifold_normals(pts_s, tris_s)
    ct, nt, mt = varifold_normals(pts_t, tris_t)
    ktau_s = K.convolve(cs, cs, ms, sigma)
    gk_s = K.grad_varlin(cs, cs, ms, sigma)        # (nf, 6, 3)
    ktau_t = K.convolve(cs, ct, mt, sigma)
    gk_t = K.grad_varlin(cs, ct, mt, sigma)
    p = pts_s
    grad = np.zeros_like(p)
    i0, i1, i2 = tris_s[:, 0], tris_s[:, 1], tris_s[:, 2]
    e0, e1, e2 = p[i2] - p[i1], p[i0] - p[i2], p[i1] - p[i0]
    mag2 = np.sum(ns * ns, axis=1)
    ok = mag2 > 1e-20
    kt = 2.0 * special_product(ktau_s - ktau_t, ns)
    aux = special_product(ms, kt)
    kt = (kt - aux / (2 * mag2[:, None])) / np.sqrt(mag2)[:, None]
    delta = gk_s - gk_t
    gk = np.stack([np.sum(special_product(delta[:, :, pdir], ns) * ns, axis=1) for pdir in range(3)],
                  axis=1) * (2.0 / 3.0)
    kt[~ok] = 0.0
    gk[~ok] = 0.0
    for idx, e in ((i0, e0), (i1, e1), (i2, e2)):
        np.add.at(grad, idx, np.cross(e, kt) + gk)
    return grad


# ---- curves (polylines of 2-point segments), d = 2 or 3 ----

def centers_tangents(pts, segs):
    """OrientedPolyLine::UpdateCentersTangents: c = (p0 + p1) / 2, t = p1 - p0."""
    p0, p1 = pts[segs[:, 0]], pts[segs[:, 1]]
    return (p0 + p1) / 2.0, p1 - p0


def curve_currents_match(K: OracleLib, sigma, pts_s, segs_s, pts_t, segs_t):
    """OrientedPolyLine::ComputeMatch: |T|^2 + |S|^2 - 2 <S, T> with tangent weights."""
    cs, ts = centers_tangents(pts_s, segs_s)
    ct, tt = centers_tangents(pts_t, segs_t)
    m = currents_norm(K, sigma, ct, tt) + currents_norm(K, sigma, cs, ts)
    return m - 2.0 * float(np.sum(K.convolve(ct, cs, ts, sigma) * tt))


def curve_currents_match_gradient(K: OracleLib, sigma, pts_s, segs_s, pts_t, segs_t):
    """OrientedPolyLine::ComputeMatchGradient: per segment Ktau = 2 (K_S t_S - K_T t_T)(c) goes
    with - / + to the two ends, and the alpha-gradient difference to both ends."""
    cs, ts = centers_tangents(pts_s, segs_s)
    ct, tt = centers_tangents(pts_t, segs_t)
    ktau = 2.0 * (K.convolve(cs, cs, ts, sigma) - K.convolve(cs, ct, tt, sigma))
    gk = K.grad_alpha(cs, cs, ts, sigma, ts) - K.grad_alpha(cs, ct, tt, sigma, ts)
    grad = np.zeros_like(pts_s)
    np.add.at(grad, segs_s[:, 0], -ktau + gk)
    np.add.at(grad, segs_s[:, 1], ktau + gk)
    return grad


def curve_varifold_tangents(pts, segs):
    """NonOrientedPolyLine::UpdateCentersTangents, :266-300: t / sqrt(|t| + 1e-20) and the
    upper-triangle products t_p t_q (p <= q)."""
    c, t = centers_tangents(pts, segs)
    t = t / np.sqrt(np.linalg.norm(t, axis=1) + 1e-20)[:, None]
    d = t.shape[1]
    iu = np.triu_indices(d)
    return c, t, (t[:, :, None] * t[:, None, :])[:, iu[0], iu[1]]


def curve_varifold_match(K: OracleLib, sigma, pts_s, segs_s, pts_t, segs_t):
    """NonOrientedPolyLine::ComputeMatch, :125-170."""
    cs, ts, ms = curve_varifold_tangents(pts_s, segs_s)
    ct, tt, mt = curve_varifold_tangents(pts_t, segs_t)
    m = varifold_norm(K, sigma, ct, tt, mt) + varifold_norm(K, sigma, cs, ts, ms)
    sdt = K.convolve(ct, cs, ms, sigma)
    return m - 2.0 * float(np.sum(tt * special_product(sdt, tt)))


def curve_varifold_match_gradient(K: OracleLib, sigma, pts_s, segs_s, pts_t, segs_t):
    """NonOrientedPolyLine::ComputeMatchGradient, :174-256."""
    cs, ts, ms = curve_varifold_tangents(pts_s, segs_s)
    ct, tt, mt = curve_varifold_tangents(pts_t, segs_t)
    d = ts.shape[1]
    ktau_s = K.convolve(cs, cs, ms, sigma)
    gk_s = K.grad_varlin(cs, cs, ms, sigma)  # (nf, d(d+1)/2, d)
    ktau_t = K.convolve(cs, ct, mt, sigma)
    gk_t = K.grad_varlin(cs, ct, mt, sigma)
    mag2 = np.sum(ts * ts, axis=1)
    ok = mag2 > 1e-20
    kt = 4.0 * special_product(ktau_s - ktau_t, ts)
    aux = special_product(ms, kt)
    kt = (kt - aux / (2 * mag2[:, None])) / np.sqrt(mag2)[:, None]
    delta = gk_s - gk_t
    gk = np.stack([np.sum(special_product(delta[:, :, q], ts) * ts, axis=1) for q in range(d)], axis=1)
    kt[~ok] = 0.0
    gk[~ok] = 0.0
    grad = np.zeros_like(pts_s)
    np.add.at(grad, segs_s[:, 0], -kt + gk)
    np.add.at(grad, segs_s[:, 1], kt + gk)
    return grad


def point_weights(pts, w):
    """PointCloud::UpdatePointWeights, :204-225: the point-data scalars, unit weights without them."""
    return np.ones(len(pts)) if w is None else np.asarray(w, dtype=np.float64).reshape(-1)


def pointcloud_match(K: OracleLib, sigma, pts_s, w_s, pts_t, w_t):
    """PointCloud::ComputeMatch, :104-146: |T|^2 + |S|^2 - 2 sum_i (K_S w_S)(t_i) w_T,i, the norms
    sum_i w_i (K w)(p_i) (UpdateSelfNorm, :229-250). The "cells" of a point cloud are its weights."""
    ws, wt = point_weights(pts_s, w_s), point_weights(pts_t, w_t)
    m = float(np.sum(K.convolve(pts_t, pts_t, wt[:, None], sigma)[:, 0] * wt))
    m += float(np.sum(K.convolve(pts_s, pts_s, ws[:, None], sigma)[:, 0] * ws))
    sdt = K.convolve(pts_t, pts_s, ws[:, None], sigma)[:, 0]
    return m - float(np.sum(sdt * (2.0 * wt)))


def pointcloud_match_gradient(K: OracleLib, sigma, pts_s, w_s, pts_t, w_t, exact: bool = False):
    """PointCloud::ComputeMatchGradient, :150-198: 2 (G_S + G_T), G_X = ConvolveGradient(S, w_S)
    with sources X and their weights. The reference adds the target term; the derivative of the
    match subtracts it (exact=True)."""
    ws, wt = point_weights(pts_s, w_s), point_weights(pts_t, w_t)
    g_s = K.grad_alpha(pts_s, pts_s, ws[:, None], sigma, ws[:, None])
    g_t = K.grad_alpha(pts_s, pts_t, wt[:, None], sigma, ws[:, None])
    return (g_s - g_t) * 2.0 if exact else (g_s + g_t) * 2.0


def volume_centers(pts, cells):
    """OrientedVolumeMesh::UpdateCentersNormals, :299-335: c = mean of the d + 1 vertices (summed in
    cell order), volume = |det(p_1 - p_0, ..., p_d - p_0)| / (6 in 3-D, 2 in 2-D); also returns
    the sign of the determinant."""
    d = pts.shape[1]
    c = pts[cells[:, 0]].copy()
    for k in range(1, d + 1):
        c += pts[cells[:, k]]
    c /= d + 1.0
    edges = np.stack([pts[cells[:, k]] - pts[cells[:, 0]] for k in range(1, d + 1)], axis=1)
    det = np.linalg.det(edges)
    return c, np.abs(det) / (6.0 if d == 3 else 2.0), np.where(det < 0, -1.0, 1.0)


def volume_match(K: OracleLib, sigma, pts_s, cells_s, pts_t, cells_t):
    """OrientedVolumeMesh::ComputeMatch, :115-155: |T|^2 + |S|^2 - 2 sum_j V_T,j (K_S V_S)(c_T,j)."""
    cs, vs, _ = volume_centers(pts_s, cells_s)
    ct, vt, _ = volume_centers(pts_t, cells_t)
    m = currents_norm(K, sigma, ct, vt[:, None]) + currents_norm(K, sigma, cs, vs[:, None])
    return m - 2.0 * float(np.sum(K.convolve(ct, cs, vs[:, None], sigma)[:, 0] * vt))


# the reference scales the 3-D volume term by the single-precision constant 1.0f / 3.0f
THIRD_F32 = float(np.float32(1.0) / np.float32(3.0))


def volume_corner_vectors(pts, cells):
    """d det / d p_k of every cell, written as OrientedVolumeMesh::ComputeMatchGradient does
    (:214-227 in 3-D, :254-266 in 2-D): (ncells, d + 1, d)."""
    d = pts.shape[1]
    p = [pts[cells[:, k]] for k in range(d + 1)]
    if d == 3:
        return np.stack([np.cross(p[3] - p[1], p[2] - p[1]), np.cross(p[2] - p[0], p[3] - p[0]),
                         np.cross(p[3] - p[0], p[1] - p[0]), np.cross(p[1] - p[0], p[2] - p[0])], axis=1)
    def perp(a, b):  # (a_y - b_y, b_x - a_x)
        return np.stack([a[:, 1] - b[:, 1], b[:, 0] - a[:, 0]], axis=1)
    return np.stack([perp(p[1], p[2]), perp(p[2], p[0]), perp(p[0], p[1])], axis=1)


def volume_match_gradient(K: OracleLib, sigma, pts_s, cells_s, pts_t, cells_t, exact: bool = False):
    """OrientedVolumeMesh::ComputeMatchGradient, :159-280: per cell Ktau = K_S V_S - K_T V_T at its
    centre times d det / d p_k (times 1.0f/3.0f in 3-D) to every corner k, and
    (G_S - G_T) / ((d + 1) / 2) to every corner, G_X = ConvolveGradient(c_S, V_S) with sources X.
    The reference drops the sign of the determinant its volumes take the absolute value of; exact=True
    keeps it (the two agree on positively oriented cells)."""
    d = pts_s.shape[1]
    cs, vs, sg = volume_centers(pts_s, cells_s)
    ct, vt, _ = volume_centers(pts_t, cells_t)
    ktau = K.convolve(cs, cs, vs[:, None], sigma)[:, 0] - K.convolve(cs, ct, vt[:, None], sigma)[:, 0]
    gk = (K.grad_alpha(cs, cs, vs[:, None], sigma, vs[:, None])
          - K.grad_alpha(cs, ct, vt[:, None], sigma, vs[:, None])) / ((d + 1.0) / 2.0)
    if exact:
        ktau = ktau * sg
    vk = volume_corner_vectors(pts_s, cells_s)
    grad = np.zeros_like(pts_s)
    for f in range(len(cells_s)):  # cell order, as the reference accumulates
        for k in range(d + 1):
            v = cells_s[f, k]
            grad[v] += (THIRD_F32 * vk[f, k] * ktau[f]) if d == 3 else vk[f, k] * ktau[f]
            grad[v] += gk[f]
    return grad


def landmark_match(K, sigma, pts_s, cells_s, pts_t, cells_t):
    """Landmark::ComputeMatch, :288-304: squared Frobenius norm of S - T (same point count)."""
    if pts_s.shape != pts_t.shape:
        raise ValueError("landmark objects need the same number of points")
    return float(np.sum((pts_s - pts_t) ** 2))


def landmark_match_gradient(K, sigma, pts_s, cells_s, pts_t, cells_t):
    """Landmark::ComputeMatchGradient, :306-322: 2 (S - T)."""
    return (pts_s - pts_t) * 2.0


KINDS = {
    "currents": (currents_match, currents_match_gradient),
    "varifold": (varifold_match, varifold_match_gradient),
    "curve_currents": (curve_currents_match, curve_currents_match_gradient),
    "curve_varifold": (curve_varifold_match, curve_varifold_match_gradient),
    "pointcloud": (pointcloud_match, pointcloud_match_gradient),
    "volume": (volume_match, volume_match_gradient),
    "landmark": (landmark_match, landmark_match_gradient),
}
