"""End-to-end parity with the reference's functional test 8 (tests/functional_tests/configure.ini
[Test8]: atlas/landmark/2d/parabola -- a DeterministicAtlas of three subjects with a two-object
template, "line" and "wave", both OrientedPolyline with data kernel width 0.2 and data-sigma 1;
deformation kernel width 0.2, 10 time points; FastGradientAscent over control points, template
and momenta from step 1e-3 for 10 iterations; tolerance 1e-8), CPU part: the FP64 oracle of the
whole estimation against the final state the reference stored (tests/golden/parabola_atlas.npz,
decoded by tests/golden/make_golden.py).

Two behaviours of the reference run are needed to reproduce it, and both are restated:
* the template-gradient smoothing width is 1 x the deformation kernel width, the default ratio,
  because the test's smoothing-kernel-width-ratio element is not the key the reference's XML
  converter reads (XmlConfigurationConverter.cxx:228 reads smoothing-kernel-with-ratio);
* every evaluation deforms the template of the previous SetFixedEffects call
  (AbstractAtlas.cxx:52-65 stores the template data it read before assigning the new map), while
  the gradient smoothing and the step use the current template (oracle.optimize.LaggedTemplate).
Without the lag the history departs from the stored one at iteration 2 (by 0.7 %).
"""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN


@pytest.fixture(scope="module")
def pb():
    return dict(np.load(os.path.join(GOLDEN, "parabola_atlas.npz")))


def parabola_problem(pb):
    objects = [dict(kind="curve_currents", cells=pb[f"tmpl{i}_segs"], sigma=float(pb["data_kernel_width"]),
                    sigma2=float(pb["data_sigma2"]), n=len(pb[f"tmpl{i}_pts"])) for i in (1, 2)]
    subjects = [[(pb[f"subj{s}_obj{i}_pts"], pb[f"subj{s}_obj{i}_segs"]) for i in (1, 2)] for s in (1, 2, 3)]
    tmpl = np.concatenate([pb["tmpl1_pts"], pb["tmpl2_pts"]])
    return objects, subjects, tmpl


def run_oracle(pb, lag=True, max_iterations=None):
    import oracle
    from oracle.optimize import LaggedTemplate, fast_gradient_ascent, multi_object_atlas_evaluator
    K = oracle.load("port")
    objects, subjects, tmpl = parabola_problem(pb)
    cp0 = pb["cp0"]
    lt = LaggedTemplate(tmpl, 1) if lag else None
    ev = multi_object_atlas_evaluator(K, objects, subjects, int(pb["number_of_time_points"]), float(pb["kernel_width"]),
                                      heun=False, smoothing_width=float(pb["smoothing_width"]), lag=lt)
    return fast_gradient_ascent(ev, [cp0, tmpl, np.zeros((len(subjects),) + cp0.shape)], float(pb["initial_step"]),
                                int(max_iterations or pb["max_iterations"]), set_fixed=lt.set_fixed if lag else None)


def test_control_point_grid(pb):
    """40 control points: the reference's grid of spacing 0.2 over the box of both objects'
    segment centres."""
    assert pb["cp0"].shape == pb["state_control_points"].shape == (40, 2)


def test_oracle_reproduces_parabola_state(pb):
    r = run_oracle(pb)
    rel = lambda a, b: np.abs(np.asarray(a) - b).max() / max(np.abs(b).max(), 1e-300)
    assert rel(r["history"], pb["state_history"]) <= 1e-10
    assert rel(r["params"][0], pb["state_control_points"]) <= 1e-10
    assert rel(r["params"][1], pb["state_template"]) <= 1e-10
    assert rel(r["params"][2], pb["state_momenta"]) <= 1e-10
    assert rel(r["aux"][1], pb["state_aux_template"]) <= 1e-10
    assert rel(r["grads"][0], pb["state_grad_control_points"]) <= 1e-10
    assert rel(r["grads"][1], pb["state_grad_template"]) <= 1e-10
    assert rel(r["grads"][2], pb["state_grad_momenta"]) <= 1e-10
    assert rel(r["step"], pb["state_step"]) <= 1e-12
    assert rel(r["grad_sq_norms"], pb["state_grad_sq_norms"]) <= 1e-10
    assert r["tau"] == pytest.approx(float(pb["state_tau"]), rel=1e-14)
    assert r["iter"] == int(pb["state_iter"]) and r["freeze_counter"] == int(pb["state_freeze_counter"])


def test_without_the_lag_the_history_departs(pb):
    r = run_oracle(pb, lag=False, max_iterations=2)
    h = pb["state_history"]
    assert np.abs(r["history"][1] - h[1]).max() <= 1e-12 * np.abs(h[1]).max()
    assert abs(r["history"][2][0] - h[2][0]) > 1e-3 * abs(h[2][0])


@pytest.fixture(scope="module")
def bn():
    return dict(np.load(os.path.join(GOLDEN, "banana_atlas.npz")))


def banana_run(bn, lag=True, max_iterations=None):
    """The reference's functional test 2 (atlas/landmark/3d/banana): a DeterministicAtlas of three
    banana surfaces (OrientedSurfaceMesh currents, data kernel 0.5, data-sigma 0.5), deformation
    kernel 1 over 20 time points, control points on the 0.3 grid, estimated by the reference's
    GradientAscent (150 iterations, 20 line-search iterations, step expand 2)."""
    import oracle
    from oracle.optimize import LaggedTemplate, atlas_evaluator, gradient_ascent
    K = oracle.load("port")
    subjects = [(bn[f"subj{i}_pts"], bn[f"subj{i}_tris"]) for i in (1, 2, 3)]
    lt = LaggedTemplate(bn["tmpl_pts"], 1) if lag else None
    ev = atlas_evaluator(K, bn["tmpl_tris"], subjects, int(bn["number_of_time_points"]), float(bn["kernel_width"]),
                         float(bn["data_kernel_width"]), float(bn["data_sigma2"]), "currents", False,
                         float(bn["smoothing_width"]), True, True, cp=bn["cp0"], tmpl=bn["tmpl_pts"], lag=lt)
    return gradient_ascent(ev, [bn["cp0"], bn["tmpl_pts"], np.zeros((3,) + bn["cp0"].shape)], float(bn["initial_step"]),
                           int(max_iterations or bn["max_iterations"]), int(bn["max_line_search"]),
                           expand=float(bn["expand"]), set_fixed=lt.set_fixed if lag else None)


def test_oracle_reproduces_banana_state(bn):
    """Every stored field: the history (9 rows; the line search fails at iteration 9, as in the
    reference's run), the final steps, the fixed effects, the momenta and the gradients."""
    r = banana_run(bn)
    rel = lambda a, b: np.abs(np.asarray(a) - b).max() / max(np.abs(b).max(), 1e-300)
    assert r["stopped"] == "line_search" and r["iter"] == int(bn["state_iter"])
    assert rel(r["history"], bn["state_history"]) <= 1e-10
    assert rel(r["step"], bn["state_step"]) <= 1e-12
    assert rel(r["params"][0], bn["state_control_points"]) <= 1e-10
    assert rel(r["params"][1], bn["state_template"]) <= 1e-10
    assert rel(r["params"][2], bn["state_momenta"]) <= 1e-10
    assert rel(r["grads"][0], bn["state_grad_control_points"]) <= 1e-9
    assert rel(r["grads"][1], bn["state_grad_template"]) <= 1e-9
    assert rel(r["grads"][2], bn["state_grad_momenta"]) <= 1e-9


def test_banana_needs_the_lag(bn):
    r = banana_run(bn, lag=False, max_iterations=2)
    h = bn["state_history"]
    assert np.abs(r["history"][1] - h[1]).max() <= 1e-12 * np.abs(h[1]).max()
    assert abs(r["history"][2][0] - h[2][0]) > 1e-2 * abs(h[2][0])
