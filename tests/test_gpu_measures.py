"""GPU parity of the point-cloud (PointCloud.cxx:104-198), volume-mesh (OrientedVolumeMesh.cxx:
115-280) and landmark (Landmark.cxx:288-322) data terms against the FP64 oracle, in both precision
modes and both gradient modes, on the reference's volume unit-test meshes
(tests/golden/volume_meshes.npz) and seeded point clouds; and registrations driven by them."""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN, normwise_rel

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


@pytest.fixture(scope="module")
def meshes():
    return dict(np.load(os.path.join(GOLDEN, "volume_meshes.npz")))


MODES = ("F64", 1e-12, 1e-11), ("F32C", 1e-6, 2e-5)


def _ctx(gb, mode, exact):
    ctx = gb.Context(mode=gb.GBK_MODE_F64 if mode == "F64" else gb.GBK_MODE_F32C)
    ctx.set_gradient_mode(gb.GBK_GRADIENT_EXACT if exact else gb.GBK_GRADIENT_REFERENCE)
    return ctx


@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("d", [2, 3])
def test_volume_term_matches_oracle(gb, K, meshes, d, exact):
    from oracle import geometry as G
    from deformetrica_code_gb300 import deformation as D
    src, tgt = ("VolumeCube", "VolumeBall") if d == 3 else ("VolumeSquare", "VolumeDisk")
    ps, cs = meshes[f"{src}_pts"], meshes[f"{src}_cells"].copy()
    pt, ct = meshes[f"{tgt}_pts"], meshes[f"{tgt}_cells"]
    if exact:
        cs[::3, [0, 1]] = cs[::3, [1, 0]]  # some negatively oriented cells
    sigma = float(meshes["kernel_width"])
    rm = G.volume_match(K, sigma, ps, cs, pt, ct)
    rg = G.volume_match_gradient(K, sigma, ps, cs, pt, ct, exact=exact)
    scale = G.volume_match(K, sigma, ps, cs, ps + 1e4, cs)
    for mode, tol_m, tol_g in MODES:
        ctx = _ctx(gb, mode, exact)
        m, g = D.volume_match(ps, cs, pt, ct, sigma, context=ctx)
        assert abs(m - rm) <= tol_m * scale, (mode, m, rm)
        assert normwise_rel(g, rg) <= tol_g, (mode, normwise_rel(g, rg))
        m2, g2 = D.volume_match(ps, cs, pt, ct, sigma, grad=False, context=ctx)
        assert m2 == m and g2 is None


@pytest.mark.parametrize("exact", [False, True])
@pytest.mark.parametrize("d", [2, 3])
def test_pointcloud_term_matches_oracle(gb, K, d, exact):
    from oracle import geometry as G
    from deformetrica_code_gb300 import deformation as D
    rng = np.random.default_rng(70 + d)
    ps, pt = rng.normal(size=(700, d)), rng.normal(size=(530, d)) + 0.3
    ws, wt = rng.uniform(0.5, 2.0, 700), rng.uniform(0.5, 2.0, 530)
    for w_s, w_t in ((ws, wt), (None, None)):
        rm = G.pointcloud_match(K, 0.6, ps, w_s, pt, w_t)
        rg = G.pointcloud_match_gradient(K, 0.6, ps, w_s, pt, w_t, exact=exact)
        scale = G.pointcloud_match(K, 0.6, ps, w_s, ps + 1e4, w_s)
        for mode, tol_m, tol_g in MODES:
            m, g = D.pointcloud_match(ps, w_s, pt, w_t, 0.6, context=_ctx(gb, mode, exact))
            assert abs(m - rm) <= tol_m * scale, (mode, m, rm)
            assert normwise_rel(g, rg) <= tol_g, (mode, normwise_rel(g, rg))


def test_pointcloud_example_sets(gb, K, meshes):
    """The 2-D point-cloud example's two 4-point sets at its object kernel width 30."""
    from oracle import geometry as G
    from deformetrica_code_gb300 import deformation as D
    s, t = meshes["sourcePoints_pts"], meshes["targetPoints_pts"]
    m, g = D.pointcloud_match(s, None, t, None, 30.0, context=_ctx(gb, "F64", False))
    assert m == pytest.approx(G.pointcloud_match(K, 30.0, s, None, t, None), rel=1e-12, abs=1e-12)
    assert normwise_rel(g, G.pointcloud_match_gradient(K, 30.0, s, None, t, None)) <= 1e-12


def test_landmark_term(gb, K, meshes):
    from deformetrica_code_gb300 import deformation as D
    rng = np.random.default_rng(5)
    for s, t in ((meshes["sourcePoints_pts"], meshes["targetPoints_pts"]),
                 (rng.normal(size=(1000, 3)), rng.normal(size=(1000, 3)))):
        m, g = D.landmark_match(s, t, context=gb.Context(mode=gb.GBK_MODE_F64))
        assert m == pytest.approx(float(np.sum((s - t) ** 2)), rel=1e-13)
        np.testing.assert_array_equal(g, 2.0 * (s - t))


def test_bad_arguments(gb, meshes):
    from deformetrica_code_gb300 import deformation as D
    ctx = gb.Context()
    ps, cs = meshes["VolumeSquare_pts"], meshes["VolumeSquare_cells"].copy()
    bad = cs.copy()
    bad[0, 0] = 10_000
    with pytest.raises(gb.GBKError):
        D.volume_match(ps, bad, ps, cs, 1.0, context=ctx)
    with pytest.raises(ValueError):
        D.landmark_match(ps, ps[:5], context=ctx)
    with pytest.raises(ValueError):
        D.pointcloud_match(ps, np.ones(3), ps, None, 1.0, context=ctx)
    with pytest.raises(gb.GBKError):
        ctx.set_gradient_mode(7)


def _registration_case(kind, meshes, rng):
    from oracle.optimize import initial_control_points
    if kind == "volume":
        tp, tc = meshes["VolumeSquare_pts"] * 10.0, meshes["VolumeSquare_cells"]
        gp, gc = meshes["VolumeDisk_pts"] * 10.0, meshes["VolumeDisk_cells"]
        return tp, tc, gp, gc, None, None, initial_control_points(tp, 5.0), 6.0, 4.0
    tp = rng.normal(0, 5, (120, 3))
    gp = tp + rng.normal(0, 1, (120, 3)) + 1.0 if kind == "landmark" else rng.normal(0, 5, (90, 3)) + 1.0
    wt = (rng.uniform(0.5, 1.5, 120), rng.uniform(0.5, 1.5, len(gp))) if kind == "pointcloud" else (None, None)
    return tp, None, gp, None, wt[0], wt[1], initial_control_points(tp, 6.0), 6.0, 5.0


@pytest.mark.parametrize("kind", ["pointcloud", "volume", "landmark"])
def test_registration_with_measure_terms(gb, K, meshes, kind):
    from oracle.deformation import registration
    from deformetrica_code_gb300 import deformation as D
    rng = np.random.default_rng(91)
    tp, tc, gp, gc, wt, wg, cp, sdef, sdata = _registration_case(kind, meshes, rng)
    mom = rng.normal(0, 0.5, cp.shape)
    L, g_cp, g_mom, info = registration(K, cp, mom, tp, wt if kind == "pointcloud" else tc, gp,
                                        wg if kind == "pointcloud" else gc, 6, sdef, sdata, 0.5, kind=kind,
                                        heun=False)
    for mode, tol in (("F64", 1e-10), ("F32C", 1e-4)):
        ctx = _ctx(gb, mode, False)
        r = D.Registration(len(cp), tp, tc, gp, gc, 6, sdef, sdata, 0.5, kind=kind, heun=False, context=ctx,
                           tmpl_weights=wt, tgt_weights=wg)
        for _ in range(3):  # eager, capture, replay
            ll, gcp, gmom = r.step(cp, mom)
            assert abs(ll[0] - L) <= tol * abs(L), (mode, ll[0], L)
            assert abs(ll[3] - info["match"]) <= tol * abs(info["match"]) + 1e-300
            assert normwise_rel(gcp, g_cp) <= 10 * tol and normwise_rel(gmom, g_mom) <= 10 * tol
        r.close()


def test_registration_point_weights_update(gb, K):
    """set_point_weights after the iteration graph exists: the replay reads the new weights."""
    from oracle.deformation import registration
    from oracle.optimize import initial_control_points
    from deformetrica_code_gb300 import deformation as D
    rng = np.random.default_rng(17)
    tp, gp = rng.normal(0, 5, (80, 2)), rng.normal(0, 5, (60, 2)) + 0.5
    cp = initial_control_points(tp, 6.0)
    mom = rng.normal(0, 0.5, cp.shape)
    r = D.Registration(len(cp), tp, None, gp, None, 5, 6.0, 4.0, 0.5, kind="pointcloud", heun=False,
                       context=_ctx(gb, "F64", False))
    for _ in range(2):
        r.step(cp, mom)
    w, wt = rng.uniform(0.5, 1.5, 80), rng.uniform(0.5, 1.5, 60)
    r.set_point_weights(w, wt)
    ll, gcp, gmom = r.step(cp, mom)
    L, g_cp, g_mom, _ = registration(K, cp, mom, tp, w, gp, wt, 5, 6.0, 4.0, 0.5, kind="pointcloud", heun=False)
    assert abs(ll[0] - L) <= 1e-10 * abs(L)
    assert normwise_rel(gmom, g_mom) <= 1e-9
    r.close()
