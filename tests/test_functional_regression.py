"""End-to-end parity with the reference's functional test 7 (tests/functional_tests/configure.ini
[Test7]: regression/landmark/2d/skulls -- a geodesic Regression of three skull curves observed at
ages 0, 3 and 5 (time indices 0, 2, 4 of 5 time points over [0, 5]), NonOrientedPolyline data term
of width 40, deformation kernel width 60, control-point spacing 40, FastGradientAscent over
control points, initial momenta and template for 10 iterations, tolerance 1e-3), CPU part: the
FP64 oracle of the whole estimation against the stored final state
(tests/golden/regression_skulls.npz), and a finite-difference check of the exact-gradient mode.

The reference's regression gradient has three properties the oracle restates
(oracle.deformation.geodesic_regression, adjoint_landmarks_jumps): the regularity gradient is
never applied (Regression::AddGradientRegularityTerm takes the gradients by value); an
observation's match gradient enters the landmark adjoint as a rate, times dt, and with the
explicit Euler scheme at most one observation is added inside the backward loop; the observation at
time index 0 is never added. The stored state is reproduced only with all three.
"""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN


@pytest.fixture(scope="module")
def rg():
    return dict(np.load(os.path.join(GOLDEN, "regression_skulls.npz")))


@pytest.fixture(scope="module")
def K():
    import oracle
    return oracle.load("port")


def regression_problem(rg):
    objects = [dict(kind="curve_varifold", cells=rg["tmpl_segs"], sigma=float(rg["data_kernel_width"]),
                    sigma2=float(rg["data_sigma2"]), n=len(rg["tmpl_pts"]))]
    observations = [[(rg[f"obs{k}_pts"], rg[f"obs{k}_segs"])] for k in range(3)]
    return objects, observations, [int(t) for t in rg["times"]]


def test_time_indices_and_grid(rg):
    T, t0, tn = int(rg["number_of_time_points"]), float(rg["t0"]), float(rg["tn"])
    ages = (0.0, 3.0, 5.0)
    idx = [int((a - t0) * ((T - 1) / (tn - t0)) + np.float32(0.5)) for a in ages]
    assert idx == list(rg["times"]) == [0, 2, 4]
    assert rg["cp0"].shape == rg["state_control_points"].shape == (16, 2)


def test_oracle_reproduces_regression_state(K, rg):
    from oracle.optimize import fast_gradient_ascent, regression_evaluator
    objects, observations, times = regression_problem(rg)
    ev = regression_evaluator(K, objects, observations, times, int(rg["number_of_time_points"]),
                              float(rg["kernel_width"]), float(rg["t0"]), float(rg["tn"]), heun=False,
                              smoothing_width=float(rg["smoothing_width"]))
    cp0 = rg["cp0"]
    r = fast_gradient_ascent(ev, [cp0, np.zeros_like(cp0), rg["tmpl_pts"]], float(rg["initial_step"]),
                             int(rg["max_iterations"]), tolerance=float(rg["tolerance"]))
    rel = lambda a, b: np.abs(np.asarray(a) - b).max() / max(np.abs(b).max(), 1e-300)
    assert rel(r["history"], rg["state_history"]) <= 1e-10
    for k, key in enumerate(("control_points", "momenta", "template")):
        assert rel(r["params"][k], rg[f"state_{key}"]) <= 1e-10
        assert rel(r["aux"][k], rg[f"state_aux_{key}"]) <= 1e-10
        assert rel(r["grads"][k], rg[f"state_grad_{key}"]) <= 1e-9
    assert rel(r["step"], rg["state_step"]) <= 1e-12
    assert rel(r["grad_sq_norms"], rg["state_grad_sq_norms"]) <= 1e-10
    assert r["tau"] == pytest.approx(float(rg["state_tau"]), rel=1e-14)
    assert r["iter"] == int(rg["state_iter"]) and r["freeze_counter"] == int(rg["state_freeze_counter"])


def test_corrected_mode_matches_finite_differences(K):
    """corrected=True on a fine time grid (T = 41, small momenta), where the O(dt) gap of the
    discretised continuous adjoint is small: central differences of the log-likelihood in the
    control points, momenta and template points of a small 2-D curve regression agree to 1 %;
    the reference's gradient, which drops the regularity term and rescales or drops observations,
    does not."""
    from oracle.deformation import geodesic_regression
    from oracle.optimize import initial_control_points
    rng = np.random.default_rng(12)
    s = np.linspace(0, np.pi, 13)
    tmpl = np.stack([np.cos(s), np.sin(s)], 1) * 2.0
    segs = np.stack([np.arange(12), np.arange(1, 13)], 1).astype(np.int32)
    obs = [[(tmpl * (1.0 + 0.05 * k) + rng.normal(0, 0.05, tmpl.shape), segs)] for k in range(3)]
    objects = [dict(kind="curve_currents", cells=segs, sigma=0.8, sigma2=0.5, n=len(tmpl))]
    cp = initial_control_points(tmpl, 1.0)
    mom = rng.normal(0, 0.05, cp.shape)
    times, T, sig = [0, 20, 40], 41, 1.2
    run = lambda c, m, t, corr: geodesic_regression(K, c, m, t, objects, obs, times, T, sig, 0.0, 1.0, False, corr)
    L = lambda c, m, t: sum(run(c, m, t, True)[:2])
    good = run(cp, mom, tmpl, True)[2:5]
    ref = run(cp, mom, tmpl, False)[2:5]
    h = 1e-5
    for which, arr in enumerate((cp, mom, tmpl)):
        fd = np.zeros_like(arr)
        for i in range(arr.shape[0]):
            for k in range(arr.shape[1]):
                a, b = [cp.copy(), mom.copy(), tmpl.copy()], [cp.copy(), mom.copy(), tmpl.copy()]
                a[which][i, k] += h
                b[which][i, k] -= h
                fd[i, k] = (L(*a) - L(*b)) / (2 * h)
        scale = np.linalg.norm(fd)
        assert np.linalg.norm(good[which] - fd) <= 1e-2 * scale, (which, np.linalg.norm(good[which] - fd) / scale)
        assert np.linalg.norm(ref[which] - fd) > 5e-2 * scale
