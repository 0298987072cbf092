"""GPU parity of multi-object templates (DeformableMultiObject): registrations whose template has
several objects with different data terms, and the multi-object atlas (gbk_mo_atlas_*) against
the oracle and against the reference's stored final state of functional test 8 (the two-object
parabola curve atlas, tests/golden/parabola_atlas.npz), including the reference's lagged template
(AbstractAtlas.cxx:52-65)."""
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
def pb():
    return dict(np.load(os.path.join(GOLDEN, "parabola_atlas.npz")))


def _parabola(pb):
    from tests.test_functional_atlas import parabola_problem
    objects, subjects, tmpl = parabola_problem(pb)
    gobj = [dict(kind="curve_currents", pts=pb[f"tmpl{i}_pts"], cells=pb[f"tmpl{i}_segs"],
                 sigma=float(pb["data_kernel_width"]), sigma2=float(pb["data_sigma2"])) for i in (1, 2)]
    return objects, subjects, tmpl, gobj


def _ctx(gb, mode):
    return gb.Context(mode=gb.GBK_MODE_F64 if mode == "F64" else gb.GBK_MODE_F32C)


def test_multi_object_registration_matches_oracle(gb, K, pb):
    from oracle.deformation import registration_multi
    from deformetrica_code_gb300 import deformation as D
    objects, subjects, tmpl, gobj = _parabola(pb)
    rng = np.random.default_rng(8)
    cp = pb["cp0"]
    mom = rng.normal(0, 0.05, cp.shape)
    d_s, r_s, g_cp, g_mom, info = registration_multi(K, cp, mom, tmpl, objects, subjects[0], 10, 0.2, heun=False)
    for mode, tol in (("F64", 1e-11), ("F32C", 1e-5)):
        r = D.Registration.from_objects(len(cp), gobj, subjects[0], 10, 0.2, heun=False, context=_ctx(gb, mode))
        for _ in range(3):
            ll, gcp, gmom = r.step(cp, mom)
            assert abs(ll[1] - d_s) <= tol * abs(d_s) and abs(ll[2] - r_s) <= tol * abs(r_s)
            assert abs(ll[3] - sum(info["matches"])) <= tol * sum(info["matches"])
            assert normwise_rel(gcp, g_cp) <= 10 * tol and normwise_rel(gmom, g_mom) <= 10 * tol
        theta = r.trajectories()["theta"][0]
        assert normwise_rel(theta, info["theta"][0]) <= 10 * tol
        r.close()


def test_mixed_object_kinds(gb, K, pb):
    """A 2-D template of a volume mesh, a weighted point cloud and landmarks, each with its own
    kernel width and data sigma."""
    from oracle.deformation import registration_multi
    from oracle.optimize import initial_control_points
    from deformetrica_code_gb300 import deformation as D
    rng = np.random.default_rng(21)
    vol = dict(np.load(os.path.join(GOLDEN, "volume_meshes.npz")))
    vp, vc = vol["VolumeSquare_pts"] * 3.0, vol["VolumeSquare_cells"]
    tp, tc = vol["VolumeDisk_pts"] * 3.0 + 0.2, vol["VolumeDisk_cells"]
    pc, pct = rng.normal(0, 2, (30, 2)), rng.normal(0, 2, (25, 2)) + 0.3
    w, wt = rng.uniform(0.5, 1.5, 30), rng.uniform(0.5, 1.5, 25)
    lmk = rng.normal(0, 2, (12, 2))
    lmt = lmk + rng.normal(0, 0.3, lmk.shape)
    oracle_objs = [dict(kind="volume", cells=vc, sigma=1.0, sigma2=0.5, n=len(vp)),
                   dict(kind="pointcloud", cells=w, sigma=1.5, sigma2=2.0, n=len(pc)),
                   dict(kind="landmark", cells=None, sigma=1.0, sigma2=0.25, n=len(lmk))]
    targets_o = [(tp, tc), (pct, wt), (lmt, None)]
    gobj = [dict(kind="volume", pts=vp, cells=vc, sigma=1.0, sigma2=0.5),
            dict(kind="pointcloud", pts=pc, cells=None, sigma=1.5, sigma2=2.0),
            dict(kind="landmark", pts=lmk, cells=None, sigma=1.0, sigma2=0.25)]
    targets_g = [(tp, tc), (pct, None), (lmt, None)]
    tmpl = np.concatenate([vp, pc, lmk])
    cp = initial_control_points(tmpl, 2.0)
    mom = rng.normal(0, 0.3, cp.shape)
    d_s, r_s, g_cp, g_mom, info = registration_multi(K, cp, mom, tmpl, oracle_objs, targets_o, 6, 2.0, heun=False)
    r = D.Registration.from_objects(len(cp), gobj, targets_g, 6, 2.0, heun=False, context=_ctx(gb, "F64"))
    r.set_point_weights(np.concatenate([np.zeros(len(vp)), w, np.zeros(len(lmk))]),
                        np.concatenate([np.zeros(len(tp)), wt, np.zeros(len(lmt))]))
    for _ in range(3):
        ll, gcp, gmom = r.step(cp, mom)
        assert abs(ll[1] - d_s) <= 1e-11 * abs(d_s)
        assert normwise_rel(gcp, g_cp) <= 1e-10 and normwise_rel(gmom, g_mom) <= 1e-10
    r.close()


@pytest.mark.parametrize("mode", ["F64", "F32C"])
def test_mo_atlas_step_matches_oracle(gb, K, pb, mode):
    from oracle.optimize import multi_object_atlas_evaluator
    from deformetrica_code_gb300 import deformation as D
    objects, subjects, tmpl, gobj = _parabola(pb)
    rng = np.random.default_rng(4)
    cp = pb["cp0"] + rng.normal(0, 0.01, pb["cp0"].shape)
    t = tmpl + rng.normal(0, 0.01, tmpl.shape)
    mom = rng.normal(0, 0.05, (3,) + cp.shape)
    ev = multi_object_atlas_evaluator(K, objects, subjects, 10, 0.2, heun=False, smoothing_width=0.2)
    terms, grads, sq = ev([cp, t, mom], True)
    a = D.MultiObjectAtlas(len(cp), gobj, subjects, 10, 0.2, heun=False, context=_ctx(gb, mode))
    a.set_template_smoothing(0.2)
    tol = 1e-11 if mode == "F64" else 1e-5
    ll, gc, gt, gm = a.step(cp, t, mom)
    assert abs(ll[1] - terms[0]) <= tol * abs(terms[0]) and abs(ll[2] - terms[1]) <= tol * abs(terms[1])
    for got, ref in zip((gc, gt, gm), grads):
        assert normwise_rel(got, ref) <= 10 * tol
    a.close()


@pytest.mark.parametrize("mode,tol", [("F64", 1e-9), ("F32C", 2e-4)])
def test_mo_atlas_reproduces_functional_test_8(gb, pb, mode, tol):
    """The whole estimation of the reference's parabola atlas: 10 FastGradientAscent iterations over
    control points, the two-object template and three subjects' momenta, with the reference's
    lagged template and smoothing width 0.2; every stored field of the final state."""
    from deformetrica_code_gb300 import deformation as D
    objects, subjects, tmpl, gobj = _parabola(pb)
    a = D.MultiObjectAtlas(40, gobj, subjects, int(pb["number_of_time_points"]), float(pb["kernel_width"]),
                           heun=False, context=_ctx(gb, mode))
    a.set_template_smoothing(float(pb["smoothing_width"]))
    r = a.optimize(pb["cp0"], tmpl, np.zeros((3, 40, 2)), int(pb["max_iterations"]), float(pb["initial_step"]))
    rel = lambda x, y: np.abs(np.asarray(x) - y).max() / np.abs(y).max()
    assert rel(r["history"], pb["state_history"]) <= tol
    assert r["freeze_counter"] == int(pb["state_freeze_counter"])
    assert rel(r["step"], pb["state_step"]) <= 1e-12
    for k, s in (("cp", "control_points"), ("template", "template"), ("mom", "momenta"),
                 ("aux_template", "aux_template"), ("grad_cp", "grad_control_points"),
                 ("grad_template", "grad_template"), ("grad_mom", "grad_momenta")):
        assert rel(r[k], pb[f"state_{s}"]) <= 10 * tol, k
    assert rel(r["grad_sq_norms"], pb["state_grad_sq_norms"]) <= 10 * tol
    assert r["tau"] == pytest.approx(float(pb["state_tau"]), rel=1e-14)
    a.close()


def test_mo_atlas_without_lag_matches_oracle(gb, K, pb):
    from oracle.optimize import fast_gradient_ascent, multi_object_atlas_evaluator
    from deformetrica_code_gb300 import deformation as D
    objects, subjects, tmpl, gobj = _parabola(pb)
    ev = multi_object_atlas_evaluator(K, objects, subjects, 10, 0.2, heun=False, smoothing_width=0.2)
    ref = fast_gradient_ascent(ev, [pb["cp0"], tmpl, np.zeros((3, 40, 2))], 1e-3, 4)
    a = D.MultiObjectAtlas(40, gobj, subjects, 10, 0.2, heun=False, context=_ctx(gb, "F64"))
    a.set_template_smoothing(0.2)
    a.set_lagged_template(False)
    r = a.optimize(pb["cp0"], tmpl, np.zeros((3, 40, 2)), 4, 1e-3)
    assert np.abs(r["history"] - ref["history"]).max() <= 1e-9 * np.abs(ref["history"]).max()
    assert normwise_rel(r["template"], ref["params"][1]) <= 1e-10
    assert r["evaluations"] == ref["evaluations"]
    a.close()


@pytest.fixture(scope="module")
def bn():
    return dict(np.load(os.path.join(GOLDEN, "banana_atlas.npz")))


@pytest.mark.parametrize("engine", ["batched", "multi_object"])
@pytest.mark.parametrize("mode,tol", [("F64", 1e-9), ("F32C", 1e-4)])
def test_reproduces_functional_test_2(gb, bn, engine, mode, tol):
    """The reference's banana atlas (three OrientedSurfaceMesh subjects) estimated by its
    GradientAscent with the lagged template, on the batched atlas and on the multi-object atlas:
    the history (the line search fails at iteration 9, as in the reference's run), the final steps
    and fixed effects."""
    from deformetrica_code_gb300 import deformation as D
    ctx = _ctx(gb, mode)
    ctx.set_estimator(gb.GBK_ESTIMATOR_GRADIENT_ASCENT)
    subjects = [(bn[f"subj{i}_pts"], bn[f"subj{i}_tris"]) for i in (1, 2, 3)]
    kw = dict(T=int(bn["number_of_time_points"]), sigma_def=float(bn["kernel_width"]), heun=False)
    if engine == "batched":
        a = D.Atlas(bn["cp0"], bn["tmpl_pts"], bn["tmpl_tris"], subjects, sigma_data=float(bn["data_kernel_width"]),
                    data_sigma2=float(bn["data_sigma2"]), kind="currents", context=ctx, **kw)
    else:
        obj = [dict(kind="currents", pts=bn["tmpl_pts"], cells=bn["tmpl_tris"], sigma=float(bn["data_kernel_width"]),
                    sigma2=float(bn["data_sigma2"]))]
        a = D.MultiObjectAtlas(len(bn["cp0"]), obj, [[s] for s in subjects], context=ctx, **kw)
    a.set_template_smoothing(float(bn["smoothing_width"]))
    r = a.optimize(bn["cp0"], bn["tmpl_pts"], np.zeros((3,) + bn["cp0"].shape), int(bn["max_iterations"]),
                   float(bn["initial_step"]), max_line_search=int(bn["max_line_search"]), expand=float(bn["expand"]))
    a.close()
    rel = lambda x, y: np.abs(np.asarray(x) - y).max() / np.abs(y).max()
    assert r["stopped"] == "line_search"
    assert r["history"].shape == bn["state_history"].shape
    assert rel(r["history"], bn["state_history"]) <= tol
    assert rel(r["step"], bn["state_step"]) <= 1e-12
    tk = "tmpl" if engine == "batched" else "template"
    assert rel(r["cp"], bn["state_control_points"]) <= 10 * tol
    assert rel(r[tk], bn["state_template"]) <= 10 * tol
    assert rel(r["mom"], bn["state_momenta"]) <= 10 * tol


def test_wrappers_reject_bad_shapes(gb, pb):
    from deformetrica_code_gb300 import deformation as D
    objects, subjects, tmpl, gobj = _parabola(pb)
    a = D.MultiObjectAtlas(40, gobj, subjects, 10, 0.2, heun=False, context=_ctx(gb, "F64"))
    with pytest.raises(ValueError):
        a.step(pb["cp0"], tmpl[:-1], np.zeros((3, 40, 2)))
    with pytest.raises(ValueError):
        a.optimize(pb["cp0"], tmpl, np.zeros((2, 40, 2)), 1)
    a.close()
    r = D.Registration.from_objects(40, gobj, subjects[0], 10, 0.2, heun=False, context=_ctx(gb, "F64"))
    with pytest.raises(ValueError):
        r.step(pb["cp0"][:-1], np.zeros((39, 2)))
    r.close()
