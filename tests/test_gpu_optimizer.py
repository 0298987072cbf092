"""GPU: the device-resident registration optimiser (gbk_registration_optimize, the reference's
FastGradientAscent.cxx:48-300) on the reference's functional test 6 (amygdala landmark
registration; see tests/test_functional_registration.py for the fixture and the oracle).

FP64 mode reproduces the final state the reference stored (log-likelihood history, control
points, momenta, the extrapolated point and its gradient, step sizes, tau, counters) to 1e-9
relative; compensated FP32 follows the same path (same accepted steps and counters) to 1e-5.
"""
import os

import numpy as np
import pytest

from tests.conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import deformetrica_code_gb300 as g
    return g


@pytest.fixture(scope="module")
def fx():
    return dict(np.load(os.path.join(GOLDEN, "amygdala_registration.npz")))


def run(gb, fx, mode):
    from deformetrica_code_gb300.deformation import Registration
    ctx = gb.Context(mode=mode)
    reg = Registration(8, fx["tmpl_pts"], fx["tmpl_tris"], fx["tgt_pts"], fx["tgt_tris"], T=10, sigma_def=10.0,
                       sigma_data=10.0, data_sigma2=0.01, kind="currents", heun=False, context=ctx)
    cp0 = fx["cp0"]
    r = reg.optimize(cp0, np.zeros_like(cp0), max_iterations=10, initial_step=1e-7)
    reg.close()
    return r


@pytest.mark.parametrize("mode_name,tol", [("f64", 1e-9), ("f32c", 1e-5)])
def test_optimizer_reproduces_reference_state(gb, fx, mode_name, tol):
    mode = gb.GBK_MODE_F64 if mode_name == "f64" else gb.GBK_MODE_F32C
    r = run(gb, fx, mode)
    h, href = r["history"], fx["state_history"]
    assert h.shape == href.shape, (h.shape, href.shape)
    assert np.all(np.abs(h - href) <= tol * np.abs(href).max() + 1e-6 * np.abs(href)), np.abs(h - href).max()
    assert r["stopped"] == "max_iterations"
    assert r["freeze_counter"] == int(fx["state_freeze_counter"])
    assert abs(r["tau"] - float(fx["state_tau"])) <= 1e-14
    np.testing.assert_allclose(r["step"], fx["state_step"], rtol=1e-14)
    np.testing.assert_allclose(r["grad_sq_norms"], fx["state_grad_sq_norms"], rtol=100 * tol)
    for key, got in (("control_points", r["cp"]), ("momenta", r["mom"]), ("aux_control_points", r["aux_cp"]),
                     ("aux_momenta", r["aux_mom"]), ("grad_control_points", r["grad_cp"]),
                     ("grad_momenta", r["grad_mom"])):
        ref = fx["state_" + key]
        rel = np.abs(got - ref).max() / np.abs(ref).max()
        assert rel <= (100 if key.startswith("grad") else 1) * tol, (key, rel)
    assert r["evaluations"] >= 21  # initial + per iteration one trial and one gradient
