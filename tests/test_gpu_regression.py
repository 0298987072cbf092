"""GPU parity of the geodesic regression (gbk_geodesic_regression_*, the reference's Regression
model) against the FP64 oracle (oracle.deformation.geodesic_regression) in both gradient modes
and both integration schemes, and against the reference's stored final state of functional test 7
(tests/golden/regression_skulls.npz)."""
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
def rg():
    return dict(np.load(os.path.join(GOLDEN, "regression_skulls.npz")))


def _problem(rg):
    from tests.test_functional_regression import regression_problem
    objects, observations, times = regression_problem(rg)
    gobj = [dict(kind="curve_varifold", pts=rg["tmpl_pts"], cells=rg["tmpl_segs"], sigma=float(rg["data_kernel_width"]),
                 sigma2=float(rg["data_sigma2"]))]
    return objects, observations, times, gobj


def _ctx(gb, mode):
    return gb.Context(mode=gb.GBK_MODE_F64 if mode == "F64" else gb.GBK_MODE_F32C)


@pytest.mark.parametrize("heun", [False, True])
@pytest.mark.parametrize("corrected", [False, True])
def test_step_matches_oracle(gb, K, rg, heun, corrected):
    from oracle.deformation import geodesic_regression
    from deformetrica_code_gb300 import deformation as D
    objects, observations, times, gobj = _problem(rg)
    rng = np.random.default_rng(3)
    cp = rg["cp0"] + rng.normal(0, 2.0, rg["cp0"].shape)
    mom = rng.normal(0, 3.0, cp.shape)
    tmpl = rg["tmpl_pts"] + rng.normal(0, 0.5, rg["tmpl_pts"].shape)
    data, reg, g_cp, g_mom, g_t, _ = geodesic_regression(K, cp, mom, tmpl, objects, observations, times, 5, 60.0, 0.0,
                                                         5.0, heun, corrected)
    sob = K.convolve(tmpl, tmpl, g_t, 60.0)
    for mode, tol in (("F64", 1e-10), ("F32C", 1e-5)):
        r = D.GeodesicRegression(len(cp), gobj, observations, times, 5, 60.0, 0.0, 5.0, heun=heun,
                                 context=_ctx(gb, mode))
        r.set_template_smoothing(60.0)
        r.set_corrected_gradient(corrected)
        for _ in range(3):  # eager, capture, replay
            ll, gc, gm, gt = r.step(cp, mom, tmpl)
            assert abs(ll[1] - data) <= tol * abs(data) and abs(ll[2] - reg) <= tol * abs(reg)
            assert normwise_rel(gc, g_cp) <= 10 * tol and normwise_rel(gm, g_mom) <= 10 * tol
            assert normwise_rel(gt, sob) <= 10 * tol
        r.close()


@pytest.mark.parametrize("mode,tol", [("F64", 1e-9), ("F32C", 1e-4)])
def test_reproduces_functional_test_7(gb, rg, mode, tol):
    """The whole estimation of the reference's skull regression: every stored field of the final
    state."""
    from deformetrica_code_gb300 import deformation as D
    objects, observations, times, gobj = _problem(rg)
    r = D.GeodesicRegression(16, gobj, observations, times, int(rg["number_of_time_points"]), float(rg["kernel_width"]),
                             float(rg["t0"]), float(rg["tn"]), heun=False, context=_ctx(gb, mode))
    r.set_template_smoothing(float(rg["smoothing_width"]))
    out = r.optimize(rg["cp0"], np.zeros_like(rg["cp0"]), rg["tmpl_pts"], int(rg["max_iterations"]),
                     float(rg["initial_step"]), tolerance=float(rg["tolerance"]))
    rel = lambda x, y: np.abs(np.asarray(x) - y).max() / np.abs(y).max()
    assert rel(out["history"], rg["state_history"]) <= tol
    assert out["freeze_counter"] == int(rg["state_freeze_counter"])
    assert rel(out["step"], rg["state_step"]) <= 1e-12
    for k, s in (("cp", "control_points"), ("mom", "momenta"), ("template", "template"), ("aux_mom", "aux_momenta"),
                 ("grad_cp", "grad_control_points"), ("grad_mom", "grad_momenta"), ("grad_template", "grad_template")):
        assert rel(out[k], rg[f"state_{s}"]) <= 10 * tol, k
    assert rel(out["grad_sq_norms"], rg["state_grad_sq_norms"]) <= 10 * tol
    assert out["tau"] == pytest.approx(float(rg["state_tau"]), rel=1e-14)
    r.close()


def test_bad_time_indices(gb, rg):
    from deformetrica_code_gb300 import deformation as D
    objects, observations, times, gobj = _problem(rg)
    with pytest.raises(gb.GBKError):
        D.GeodesicRegression(16, gobj, observations, [0, 4, 2], 5, 60.0, 0.0, 5.0, context=_ctx(gb, "F64"))
    with pytest.raises(gb.GBKError):
        D.GeodesicRegression(16, gobj, observations, [0, 2, 5], 5, 60.0, 0.0, 5.0, context=_ctx(gb, "F64"))
