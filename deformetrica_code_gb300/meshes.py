"""Synthetic triangle meshes for the benchmark and test workloads (no mesh files needed).

* icosphere(subdivisions, radius, center): 10 * 4^k + 2 vertices, 20 * 4^k faces (k = 5 gives the
  10,242-vertex / 20,480-face template of the shooting+adjoint registration workload);
* sine_bump(points, normals, amp, freq): vertex += amp sin(freq pi x) along the vertex normal
  (the registration target);
* torus(nu, nv, R, r, noise, seed): a (u, v) grid torus with 2 nu nv faces (500 x 200 -> 200,000);
* perturbed_sphere(n, noise, seed): Fibonacci points on the unit sphere perturbed radially and
  triangulated by their convex hull (2 n - 4 faces), the atlas subjects;
* tet_grid(n, noise, seed): the unit cube cut into n^3 cells of six tetrahedra each (6 n^3 cells,
  all positively oriented), vertices jittered, for the volume-mesh data term.

Faces are oriented so that the reference's face normal (p2 - p0) x (p1 - p0) / 2 points outward;
the currents data term depends on orientation (OrientedSurfaceMesh.cxx:298-328).
"""
from __future__ import annotations

import numpy as np


def icosphere(subdivisions: int = 5, radius: float = 0.4, center=(0.5, 0.5, 0.5)):
    t = (1.0 + 5 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], float)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
                  [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
                  [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)
    v /= np.linalg.norm(v, axis=1)[:, None]
    for _ in range(subdivisions):
        edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.sort(edges, axis=1)
        uniq, inv = np.unique(key, axis=0, return_inverse=True)
        mids = v[uniq[:, 0]] + v[uniq[:, 1]]
        mids /= np.linalg.norm(mids, axis=1)[:, None]
        base = v.shape[0]
        v = np.concatenate([v, mids])
        nf = f.shape[0]
        m01, m12, m20 = (base + inv[:nf], base + inv[nf:2 * nf], base + inv[2 * nf:])
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1), np.stack([m01, f[:, 1], m12], 1),
            np.stack([m20, m12, f[:, 2]], 1), np.stack([m01, m12, m20], 1)])
    pts = np.asarray(center, float) + radius * v
    return pts, orient_outward_faces(pts, f, np.asarray(center, float))


def orient_outward_faces(pts, f, center):
    """Flip faces whose normal n = (p2 - p0) x (p1 - p0) points towards `center`."""
    p0, p1, p2 = pts[f[:, 0]], pts[f[:, 1]], pts[f[:, 2]]
    n = np.cross(p2 - p0, p1 - p0)
    c = (p0 + p1 + p2) / 3.0 - center
    bad = np.sum(n * c, axis=1) < 0
    f = f.copy()
    f[bad] = f[bad][:, [0, 2, 1]]
    return f


def vertex_normals(pts, f):
    """Area-weighted vertex normals (outward for outward-oriented faces)."""
    p0, p1, p2 = pts[f[:, 0]], pts[f[:, 1]], pts[f[:, 2]]
    n = np.cross(p2 - p0, p1 - p0)
    vn = np.zeros_like(pts)
    for k in range(3):
        np.add.at(vn, f[:, k], n)
    return vn / np.maximum(np.linalg.norm(vn, axis=1)[:, None], 1e-30)


def sine_bump(pts, f, amp: float = 0.05, freq: float = 4.0):
    """vertex += amp * sin(freq * pi * x) * outward normal (x = first coordinate)."""
    return pts + amp * np.sin(freq * np.pi * pts[:, :1]) * vertex_normals(pts, f)


def torus(nu: int = 500, nv: int = 200, R: float = 0.5, r: float = 0.2, noise: float = 0.01,
          seed: int = 5, center=(0.0, 0.0, 0.0)):
    u = np.arange(nu) * (2 * np.pi / nu)
    w = np.arange(nv) * (2 * np.pi / nv)
    U, Wg = np.meshgrid(u, w, indexing="ij")
    pts = np.stack([(R + r * np.cos(Wg)) * np.cos(U), (R + r * np.cos(Wg)) * np.sin(U),
                    r * np.sin(Wg)], axis=-1).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    pts = pts + noise * rng.standard_normal(pts.shape) + np.asarray(center, float)
    i, j = np.meshgrid(np.arange(nu), np.arange(nv), indexing="ij")
    a = i * nv + j
    b = ((i + 1) % nu) * nv + j
    c = ((i + 1) % nu) * nv + (j + 1) % nv
    d = i * nv + (j + 1) % nv
    f = np.concatenate([np.stack([a, b, c], -1).reshape(-1, 3), np.stack([a, c, d], -1).reshape(-1, 3)])
    # orient against the tube centre line
    p0, p1, p2 = pts[f[:, 0]], pts[f[:, 1]], pts[f[:, 2]]
    n = np.cross(p2 - p0, p1 - p0)
    cen = (p0 + p1 + p2) / 3.0 - np.asarray(center, float)
    ang = np.arctan2(cen[:, 1], cen[:, 0])
    axis_pt = np.stack([R * np.cos(ang), R * np.sin(ang), np.zeros_like(ang)], -1)
    bad = np.sum(n * (cen - axis_pt), axis=1) < 0
    f[bad] = f[bad][:, [0, 2, 1]]
    return pts, f.astype(np.int64)


def perturbed_sphere(n: int, noise: float = 0.02, seed: int = 4, radius: float = 0.4,
                     center=(0.5, 0.5, 0.5)):
    """Fibonacci sphere with radial noise, triangulated by its convex hull (2n - 4 faces)."""
    from scipy.spatial import ConvexHull
    k = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * k / n)
    theta = np.pi * (1 + 5 ** 0.5) * k
    v = np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)], 1)
    f = ConvexHull(v).simplices.astype(np.int64)
    rng = np.random.default_rng(seed)
    pts = np.asarray(center, float) + radius * v * (1.0 + noise * rng.standard_normal((n, 1)))
    return pts, orient_outward_faces(pts, f, np.asarray(center, float))


def tet_grid(n: int = 30, noise: float = 0.1, seed: int = 7, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    """(n+1)^3 grid vertices over [lo, hi] moved by noise x cell size (uniform, seeded), and the six
    tetrahedra p0, p_a, p_ab, p7 of every cell along the monotone paths of its main diagonal, each
    ordered so that det(p1 - p0, p2 - p0, p3 - p0) > 0 (OrientedVolumeMesh's volumes)."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, float), np.asarray(hi, float)
    g = np.linspace(0.0, 1.0, n + 1)
    x, y, z = np.meshgrid(g, g, g, indexing="ij")
    pts = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    pts = pts + rng.uniform(-noise, noise, pts.shape) / n
    pts = lo + pts * (hi - lo)
    idx = lambda i, j, k: (i * (n + 1) + j) * (n + 1) + k
    i, j, k = (a.ravel() for a in np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"))
    corner = {c: idx(i + c[0], j + c[1], k + c[2]) for c in np.ndindex(2, 2, 2)}
    tets = []
    for a in range(3):
        for b in range(3):
            if a == b:
                continue
            ea = tuple(1 if t == a else 0 for t in range(3))
            eab = tuple(1 if t in (a, b) else 0 for t in range(3))
            tets.append(np.stack([corner[(0, 0, 0)], corner[ea], corner[eab], corner[(1, 1, 1)]], axis=1))
    cells = np.concatenate(tets).astype(np.int32)
    e = pts[cells[:, 1:]] - pts[cells[:, :1]]
    neg = np.linalg.det(e) < 0
    cells[neg, 1], cells[neg, 2] = cells[neg, 2].copy(), cells[neg, 1].copy()
    return pts, cells
