"""Oracle checks of the point-cloud, volume-mesh and landmark data terms (PointCloud.cxx,
OrientedVolumeMesh.cxx, Landmark.cxx), no GPU: the reference's own volume-gradient unit test
(TestVolumeGradient.cxx:86-120) restated on the oracle with its meshes (tests/golden/volume_meshes.npz),
the exact-gradient mode against finite differences, and the VTK unstructured-grid and point-data
readers."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN


@pytest.fixture(scope="module")
def K():
    import oracle
    return oracle.load("port")


@pytest.fixture(scope="module")
def meshes():
    return dict(np.load(os.path.join(GOLDEN, "volume_meshes.npz")))


def _numeric(f, pts, h, central=False):
    g = np.zeros_like(pts)
    f0 = None if central else f(pts)
    for i in range(pts.shape[0]):
        for k in range(pts.shape[1]):
            p = pts.copy()
            p[i, k] += h
            if central:
                q = pts.copy()
                q[i, k] -= h
                g[i, k] = (f(p) - f(q)) / (2 * h)
            else:
                g[i, k] = (f(p) - f0) / h
    return g


@pytest.mark.parametrize("src,tgt", [("VolumeCube", "VolumeBall"), ("VolumeSquare", "VolumeDisk")])
def test_volume_gradient_unit_test(K, meshes, src, tgt):
    """TestVolumeGradient: forward differences of step 1e-5f against ComputeMatchGradient, every
    entry within 1e-5, kernel width 1."""
    from oracle import geometry as G
    ps, cs = meshes[f"{src}_pts"], meshes[f"{src}_cells"]
    pt, ct = meshes[f"{tgt}_pts"], meshes[f"{tgt}_cells"]
    sigma, h, tol = float(meshes["kernel_width"]), float(meshes["fd_step"]), float(meshes["tolerance"])
    analytic = G.volume_match_gradient(K, sigma, ps, cs, pt, ct)
    numeric = _numeric(lambda p: G.volume_match(K, sigma, p, cs, pt, ct), ps, h)
    assert np.abs(analytic - numeric).max() <= tol
    # the meshes are positively oriented, where the reference's formula is the exact derivative
    assert np.all(G.volume_centers(ps, cs)[2] > 0)
    assert np.array_equal(analytic, G.volume_match_gradient(K, sigma, ps, cs, pt, ct, exact=True))


@pytest.mark.parametrize("d", [2, 3])
def test_volume_exact_mode_on_flipped_cells(K, meshes, d):
    """Reversed cells: the reference's formula keeps the signed-volume derivative, the exact mode
    follows the match (which uses |det|)."""
    from oracle import geometry as G
    src, tgt = ("VolumeCube", "VolumeBall") if d == 3 else ("VolumeSquare", "VolumeDisk")
    ps, cs = meshes[f"{src}_pts"], meshes[f"{src}_cells"].copy()
    pt, ct = meshes[f"{tgt}_pts"], meshes[f"{tgt}_cells"]
    cs[::3, [0, 1]] = cs[::3, [1, 0]]
    assert np.any(G.volume_centers(ps, cs)[2] < 0)
    numeric = _numeric(lambda p: G.volume_match(K, 1.0, p, cs, pt, ct), ps, 1e-6, central=True)
    exact = G.volume_match_gradient(K, 1.0, ps, cs, pt, ct, exact=True)
    ref = G.volume_match_gradient(K, 1.0, ps, cs, pt, ct)
    scale = np.abs(numeric).max()
    assert np.abs(exact - numeric).max() <= 1e-6 * scale  # 1.0f/3.0f in 3-D: 3e-8 relative
    assert np.abs(ref - numeric).max() > 1e-2 * scale


@pytest.mark.parametrize("d", [2, 3])
def test_pointcloud_gradient_modes(K, d):
    from oracle import geometry as G
    rng = np.random.default_rng(40 + d)
    ps, pt = rng.normal(size=(25, d)), rng.normal(size=(18, d)) + 0.4
    ws, wt = rng.uniform(0.5, 2.0, 25), rng.uniform(0.5, 2.0, 18)
    f = lambda p: G.pointcloud_match(K, 0.8, p, ws, pt, wt)
    numeric = _numeric(f, ps, 1e-6, central=True)
    exact = G.pointcloud_match_gradient(K, 0.8, ps, ws, pt, wt, exact=True)
    assert np.abs(exact - numeric).max() <= 1e-6 * np.abs(numeric).max()
    # the reference's formula: 2 (G_S + G_T), G_X = ConvolveGradient(S, w_S) with sources X
    g_s = K.grad_alpha(ps, ps, ws[:, None], 0.8, ws[:, None])
    g_t = K.grad_alpha(ps, pt, wt[:, None], 0.8, ws[:, None])
    np.testing.assert_array_equal(G.pointcloud_match_gradient(K, 0.8, ps, ws, pt, wt), (g_s + g_t) * 2.0)
    # unit weights without point data
    assert G.pointcloud_match(K, 0.8, ps, None, pt, None) == G.pointcloud_match(K, 0.8, ps, np.ones(25), pt,
                                                                                 np.ones(18))


def test_landmark_term(K, meshes):
    from oracle import geometry as G
    s, t = meshes["sourcePoints_pts"], meshes["targetPoints_pts"]
    assert G.landmark_match(K, 1.0, s, None, t, None) == pytest.approx(float(np.sum((s - t) ** 2)), rel=1e-15)
    np.testing.assert_array_equal(G.landmark_match_gradient(K, 1.0, s, None, t, None), 2.0 * (s - t))
    with pytest.raises(ValueError):
        G.landmark_match(K, 1.0, s, None, t[:3], None)


def test_vtk_unstructured_grid_and_point_scalars(tmp_path):
    from deformetrica_code_gb300.formats import read_vtk_polydata, read_vtk_point_weights
    f = tmp_path / "cells.vtk"
    f.write_text("# vtk DataFile Version 4.0\nvtk output\nASCII\nDATASET UNSTRUCTURED_GRID\n"
                 "POINTS 5 float\n0 0 0 1 0 0 0 1 0\n0 0 1 1 1 1\n"
                 "CELLS 2 10\n4 0 1 2 3\n4 1 2 3 4\n\nCELL_TYPES 2\n10\n10\n"
                 "POINT_DATA 5\nSCALARS w float 1\nLOOKUP_TABLE default\n0.5 1 1.5 2 2.5\n")
    p, c = read_vtk_polydata(str(f))
    assert p.shape == (5, 3) and c.tolist() == [[0, 1, 2, 3], [1, 2, 3, 4]]
    np.testing.assert_array_equal(read_vtk_point_weights(str(f)), [0.5, 1, 1.5, 2, 2.5])
    g = tmp_path / "pts.vtk"
    g.write_text("# vtk DataFile Version 3.0\nx\nASCII\nDATASET POLYDATA\nPOINTS 2 float\n0 0 0 1 1 0\n")
    assert read_vtk_point_weights(str(g)) is None
    h = tmp_path / "mismatch.vtk"
    h.write_text("# vtk DataFile Version 3.0\nx\nASCII\nDATASET POLYDATA\nPOINTS 2 float\n0 0 0 1 1 0\n"
                 "POINT_DATA 2\nSCALARS w float 3\nLOOKUP_TABLE default\n1 2 3 4 5 6\n")
    assert read_vtk_point_weights(str(h)) is None  # several components: unit weights
