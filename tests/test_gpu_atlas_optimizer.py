"""GPU: the device-resident atlas optimiser (gbk_atlas_optimize: the reference's
FastGradientAscent.cxx:48-300 over ControlPoints, TemplateData and every subject's Momenta of a
DeterministicAtlas) against the FP64 oracle (oracle.optimize.fast_gradient_ascent over
oracle.optimize.atlas_evaluator), including the smoothed template gradient
(AbstractAtlas::ConvolveGradTemplate) and its <L2, smoothed> norm, on three uneven subjects."""
import numpy as np
import pytest

from tests.conftest import normwise_rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import deformetrica_code_gb300 as g
    return g


def problem():
    from deformetrica_code_gb300 import meshes as M
    tp, tf = M.icosphere(2, 0.35)
    targets = [M.perturbed_sphere(n, noise=0.02, seed=70 + i, radius=0.37) for i, n in enumerate((150, 320, 230))]
    g = np.linspace(0.25, 0.75, 3)
    cp = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    mom = np.zeros((len(targets), cp.shape[0], 3))
    return cp, tp, tf, targets, mom, dict(T=5, sigma_def=0.25, sigma_data=0.15, data_sigma2=0.01)


@pytest.mark.parametrize("groups,lag", [((True, True), True), ((True, True), False), ((False, True), True),
                                        ((True, False), True)])
def test_atlas_optimizer_matches_oracle(gb, groups, lag):
    """lag: the reference's lagged template (AbstractAtlas.cxx:52-65, the default) or not."""
    import oracle
    from oracle.optimize import LaggedTemplate, atlas_evaluator, fast_gradient_ascent
    from deformetrica_code_gb300.deformation import Atlas
    opt_cp, opt_t = groups
    K = oracle.load("port")
    cp, tp, tf, targets, mom, kw = problem()
    smoothing, iters, step0 = 0.1, 4, 1e-3
    lt = LaggedTemplate(tp, int(opt_cp)) if lag and opt_t else None
    ev = atlas_evaluator(K, tf, targets, kw["T"], kw["sigma_def"], kw["sigma_data"], kw["data_sigma2"], "currents",
                         True, smoothing, opt_cp, opt_t, cp=cp, tmpl=tp, lag=lt)
    start = ([cp] if opt_cp else []) + ([tp] if opt_t else []) + [mom]
    ref = fast_gradient_ascent(ev, start, step0, iters, set_fixed=lt.set_fixed if lt else None)
    for mode, tol in ((gb.GBK_MODE_F64, 1e-9), (gb.GBK_MODE_F32C, 1e-5)):
        ctx = gb.Context(mode=mode)
        atlas = Atlas(cp, tp, tf, targets, kind="currents", context=ctx, **kw)
        atlas.set_template_smoothing(smoothing)
        atlas.set_lagged_template(lag)
        r = atlas.optimize(cp, tp, mom, iters, step0, optimize_cp=opt_cp, optimize_template=opt_t)
        atlas.close()
        h, hr = r["history"], ref["history"]
        assert h.shape == hr.shape, (mode, h.shape, hr.shape)
        assert np.all(np.abs(h - hr) <= tol * np.abs(hr).max() + 1e-6 * np.abs(hr)), (mode, np.abs(h - hr).max())
        assert r["freeze_counter"] == ref["freeze_counter"] and abs(r["tau"] - ref["tau"]) <= 1e-14
        np.testing.assert_allclose(r["step"], ref["step"], rtol=1e-14)
        k = 0
        if opt_cp:
            assert normwise_rel(r["cp"], ref["params"][k]) <= tol
            k += 1
        else:
            assert np.array_equal(r["cp"], cp)
        if opt_t:
            assert normwise_rel(r["tmpl"], ref["params"][k]) <= tol
            k += 1
        assert normwise_rel(r["mom"].reshape(-1, 3), ref["params"][k].reshape(-1, 3)) <= 100 * tol
        np.testing.assert_allclose(r["grad_sq_norms"], ref["grad_sq_norms"], rtol=1000 * tol)
