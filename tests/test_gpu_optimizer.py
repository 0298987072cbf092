"""GPU: the device-resident registration optimiser (gbk_registration_optimize, the reference's
FastGradientAscent.cxx:48-300) on the reference's functional tests 6 (amygdala surface
registration, 3-D currents) and 5 (skull curve registration, 2-D varifold); see
tests/test_functional_registration.py for the fixtures and the oracle.

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


CASES = {
    "amygdala": dict(file="amygdala_registration.npz", cells="tmpl_tris", tcells="tgt_tris", kind="currents"),
    "skull": dict(file="skull_registration.npz", cells="tmpl_segs", tcells="tgt_segs", kind="curve_varifold"),
}


def run(gb, case, mode):
    from deformetrica_code_gb300.deformation import Registration
    c = CASES[case]
    fx = dict(np.load(os.path.join(GOLDEN, c["file"])))
    ctx = gb.Context(mode=mode)
    cp0 = fx["cp0"]
    reg = Registration(cp0.shape[0], fx["tmpl_pts"], fx[c["cells"]], fx["tgt_pts"], fx[c["tcells"]],
                       T=int(fx["number_of_time_points"]), sigma_def=float(fx["kernel_width"]),
                       sigma_data=float(fx["data_kernel_width"]), data_sigma2=float(fx["data_sigma2"]),
                       kind=c["kind"], heun=False, context=ctx)
    r = reg.optimize(cp0, np.zeros_like(cp0), max_iterations=int(fx["max_iterations"]),
                     initial_step=float(fx["initial_step"]))
    reg.close()
    return r, fx


@pytest.mark.parametrize("case", ["amygdala", "skull"])
@pytest.mark.parametrize("mode_name,tol", [("f64", 1e-9), ("f32c", 1e-5)])
def test_optimizer_reproduces_reference_state(gb, case, mode_name, tol):
    mode = gb.GBK_MODE_F64 if mode_name == "f64" else gb.GBK_MODE_F32C
    r, fx = run(gb, case, mode)
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
