"""GPU parity of the curve data terms (OrientedPolyLine: currents with tangents; NonOrientedPolyLine:
varifold, NonOrientedPolyLine.cxx:125-300) against the FP64 oracle, in 2-D and 3-D, both precision
modes, on the reference's skull curves (functional test 5 data, tests/golden/skull_registration.npz)
and on a random 3-D lift of them."""
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
def skull():
    return dict(np.load(os.path.join(GOLDEN, "skull_registration.npz")))


@pytest.mark.parametrize("kind", ["curve_currents", "curve_varifold"])
@pytest.mark.parametrize("d", [2, 3])
def test_curve_terms_match_oracle(gb, skull, kind, d):
    import oracle
    from oracle import geometry as G
    from deformetrica_code_gb300 import deformation as D
    K = oracle.load("port")
    rng = np.random.default_rng(10 + d)
    lift = lambda p: p if d == 2 else np.concatenate([p, rng.normal(0, 5, (p.shape[0], 1))], axis=1)
    ps, pt = np.ascontiguousarray(lift(skull["tmpl_pts"])), np.ascontiguousarray(lift(skull["tgt_pts"]))
    ss, st = skull["tmpl_segs"], skull["tgt_segs"]
    fm, fg = G.KINDS[kind]
    rm, rg = fm(K, 40.0, ps, ss, pt, st), fg(K, 40.0, ps, ss, pt, st)
    scale = fm(K, 40.0, ps, ss, ps + 1e4, ss)  # |S|^2 + |S|^2: the distance to a far copy
    api = D.curve_currents_match if kind == "curve_currents" else D.curve_varifold_match
    for mode, tol_m, tol_g in ((gb.GBK_MODE_F64, 1e-11, 1e-10), (gb.GBK_MODE_F32C, 1e-6, 2e-5)):
        ctx = gb.Context(mode=mode)
        m, g = api(ps, ss, pt, st, 40.0, context=ctx)
        assert abs(m - rm) <= tol_m * scale, (mode, m, rm)
        assert normwise_rel(g, rg) <= tol_g, (mode, normwise_rel(g, rg))
