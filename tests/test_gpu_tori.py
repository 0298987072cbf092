"""GPU parity of the surface data terms on the two-tori workload (major radius 0.5, minor 0.2,
vertex noise N(0, 0.01^2), seeds 5 and 6, sigma = 0.05): currents (OrientedSurfaceMesh.cxx:124-352)
and varifold (NonOrientedSurfaceMesh.cxx:124-378) distance and vertex gradient.

* Reduced grid (60 x 24 -> 2,880 triangles a torus) against the FP64 oracle, in caller order and
  in the spatial order, both precision modes.
* Full grid (500 x 200 -> 200,000 triangles a torus), where the oracle is out of reach: the pruned
  spatial order gives the same bits as evaluating every pair, and agrees with caller order to the
  FP32 tolerance.
"""
import numpy as np
import pytest

from tests.conftest import normwise_rel

pytestmark = pytest.mark.gpu

SIGMA = 0.05


@pytest.fixture(scope="module")
def gb():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import deformetrica_code_gb300 as g
    return g


@pytest.fixture(scope="module")
def ctx(gb):
    c = gb.Context()
    yield c
    c.set_order(gb.GBK_ORDER_AUTO)
    c.set_mode(gb.GBK_MODE_F32C)


@pytest.fixture(scope="module")
def K():
    import oracle
    return oracle.load("port")


def tori(nu, nv):
    from deformetrica_code_gb300.meshes import torus
    ps, fs = torus(nu, nv, seed=5)
    pt, ft = torus(nu, nv, seed=6)
    return ps, fs, pt, ft


@pytest.mark.parametrize("kind", ["currents", "varifold"])
def test_reduced_tori_match_oracle(gb, ctx, K, kind):
    from oracle import geometry as G
    from deformetrica_code_gb300.deformation import currents_match, varifold_match
    ps, fs, pt, ft = tori(60, 24)
    fm = currents_match if kind == "currents" else varifold_match
    rm = (G.currents_match if kind == "currents" else G.varifold_match)(K, SIGMA, ps, fs, pt, ft)
    rg = (G.currents_match_gradient if kind == "currents" else G.varifold_match_gradient)(K, SIGMA, ps, fs, pt, ft)
    scale = G.currents_norm(K, SIGMA, *G.centers_normals(ps, fs)) if kind == "currents" else \
        G.varifold_norm(K, SIGMA, *G.varifold_normals(ps, fs))
    for order in (gb.GBK_ORDER_OFF, gb.GBK_ORDER_SPATIAL):
        ctx.set_order(order)
        for mode, tol_m, tol_g in ((gb.GBK_MODE_F64, 1e-10, 1e-10), (gb.GBK_MODE_F32C, 1e-5, 2e-5)):
            ctx.set_mode(mode)
            m, g = fm(ps, fs, pt, ft, SIGMA, context=ctx)
            assert abs(m - rm) <= tol_m * scale, (order, mode, m, rm)
            assert normwise_rel(g, rg) <= tol_g, (order, mode, normwise_rel(g, rg))


@pytest.mark.parametrize("kind", ["currents", "varifold"])
def test_full_tori_pruning_exact_and_order_consistent(gb, ctx, kind):
    from deformetrica_code_gb300.deformation import currents_match, varifold_match
    ps, fs, pt, ft = tori(500, 200)
    assert fs.shape[0] == 200_000 and ft.shape[0] == 200_000
    fm = currents_match if kind == "currents" else varifold_match
    ctx.set_mode(gb.GBK_MODE_F32C)
    out = {}
    for order in (gb.GBK_ORDER_SPATIAL, gb.GBK_ORDER_SPATIAL_NOPRUNE, gb.GBK_ORDER_OFF):
        ctx.set_order(order)
        p0 = ctx.evaluated_pairs()
        out[order] = fm(ps, fs, pt, ft, SIGMA, context=ctx) + (ctx.evaluated_pairs() - p0,)
    m_p, g_p, n_p = out[gb.GBK_ORDER_SPATIAL]
    m_n, g_n, n_n = out[gb.GBK_ORDER_SPATIAL_NOPRUNE]
    m_o, g_o, n_o = out[gb.GBK_ORDER_OFF]
    assert m_p == m_n and np.array_equal(g_p, g_n)
    assert n_p < n_n == n_o  # pruning skipped work; the other two evaluated every pair
    # scale of the distance: against a far copy of itself the match is 2 |S|^2 (no cross term)
    two_norm2, _ = fm(ps, fs, ps + 100.0, fs, SIGMA, grad=False, context=ctx)
    assert abs(m_p - m_o) <= 1e-5 * two_norm2
    assert normwise_rel(g_p, g_o) <= 2e-6
