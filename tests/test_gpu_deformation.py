"""GPU parity of the deformation engine, the data terms and the registration step against the FP64
oracle (oracle/deformation.py, oracle/geometry.py), which restates Diffeos.cxx,
AdjointEquationsIntegrator.cxx, OrientedSurfaceMesh.cxx and NonOrientedSurfaceMesh.cxx.

Tolerances (normwise relative error max_i |err_i| / max_i |ref_i| over a whole trajectory):
FP64 mode 1e-10; compensated FP32 mode 2e-5 (per-pass errors ~1e-7 compound over the time steps
and through the adjoint's second-order terms).
"""
import numpy as np
import pytest

from tests.conftest import normwise_rel

pytestmark = pytest.mark.gpu

F64 = 1e-10
F32 = 2e-5


@pytest.fixture(scope="module")
def gb():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import deformetrica_code_gb300 as g
    return g


@pytest.fixture(scope="module")
def ctx(gb):
    return gb.Context()


@pytest.fixture(scope="module")
def K():
    import oracle
    return oracle.load("port")


def grid_cp(k=4, lo=0.2, hi=0.8, d=3):
    g = np.linspace(lo, hi, k)
    return np.stack(np.meshgrid(*([g] * d), indexing="ij"), -1).reshape(-1, d)


def small_problem(d=3, seed=0):
    rng = np.random.default_rng(seed)
    cp = grid_cp(4 if d == 3 else 6, d=d)
    mom = 0.05 * rng.standard_normal(cp.shape)
    lm = rng.uniform(0.2, 0.8, (150, d))
    return cp, mom, lm


def modes(gb):
    return [(gb.GBK_MODE_F64, F64), (gb.GBK_MODE_F32C, F32)]


@pytest.mark.parametrize("d", [2, 3])
def test_shoot_flow_adjoints_match_oracle(gb, ctx, K, d):
    from oracle import deformation as D
    from deformetrica_code_gb300.deformation import Deformation
    cp, mom, lm0 = small_problem(d, seed=d)
    sigma, T = 0.3, 6
    pos_r, mom_r = D.shoot(K, sigma, cp, mom, T)
    lm_r = D.flow_landmarks(K, sigma, pos_r, mom_r, lm0, heun=True)
    th_T = np.random.default_rng(7).standard_normal(lm0.shape)
    th_r = D.adjoint_landmarks(K, sigma, pos_r, mom_r, lm_r, th_T, heun=True)
    xp_r, xm_r = D.adjoint_diffeo(K, sigma, pos_r, mom_r, lm_r, th_r, heun=True)
    for mode, tol in modes(gb):
        ctx.set_mode(mode)
        df = Deformation(d, sigma, T, heun=True, context=ctx)
        pos, mo = df.shoot(cp, mom)
        assert normwise_rel(pos.reshape(-1, d), np.concatenate(pos_r)) <= tol
        assert normwise_rel(mo.reshape(-1, d), np.concatenate(mom_r)) <= tol
        lm = df.flow(pos, mo, lm0)
        assert normwise_rel(lm.reshape(-1, d), np.concatenate(lm_r)) <= tol
        th = df.adjoint_landmarks(pos, mo, lm, th_T)
        assert normwise_rel(th.reshape(-1, d), np.concatenate(th_r)) <= tol
        xp, xm = df.adjoint_diffeo(pos, mo, lm, th)
        assert normwise_rel(xp.reshape(-1, d), np.concatenate(xp_r)) <= tol
        assert normwise_rel(xm.reshape(-1, d), np.concatenate(xm_r)) <= tol


def test_euler_flow_without_heun(gb, ctx, K):
    from oracle import deformation as D
    from deformetrica_code_gb300.deformation import Deformation
    cp, mom, lm0 = small_problem(3, seed=4)
    pos_r, mom_r = D.shoot(K, 0.25, cp, mom, 5)
    lm_r = D.flow_landmarks(K, 0.25, pos_r, mom_r, lm0, heun=False)
    ctx.set_mode(gb.GBK_MODE_F64)
    df = Deformation(3, 0.25, 5, heun=False, context=ctx)
    pos, mo = df.shoot(cp, mom)
    assert normwise_rel(df.flow(pos, mo, lm0).reshape(-1, 3), np.concatenate(lm_r)) <= F64


def test_compute_update_at_fused_equals_seven_calls(gb, ctx, K):
    """The fused CP x CP pass reproduces the reference's five CP kernel calls + two landmark calls
    of ComputeUpdateAt (AdjointEquationsIntegrator.cxx:476-570)."""
    from oracle import deformation as D
    from deformetrica_code_gb300.deformation import Deformation
    rng = np.random.default_rng(11)
    for d in (2, 3):
        cp = rng.uniform(0.2, 0.8, (57, d))
        mom, xp, xm = (rng.standard_normal((57, d)) for _ in range(3))
        lm, th = rng.uniform(0.1, 0.9, (91, d)), rng.standard_normal((91, d))
        for with_lm in (False, True):
            ref = D.compute_update_at(K, 0.35, cp, mom, xp, xm, lm if with_lm else None, th if with_lm else None)
            for mode, tol in modes(gb):
                ctx.set_mode(mode)
                df = Deformation(d, 0.35, 2, context=ctx)
                got = df.compute_update_at(cp, mom, xp, xm, lm if with_lm else None, th if with_lm else None)
                for g_, r_ in zip(got, ref):
                    assert normwise_rel(g_, r_) <= (tol if mode == gb.GBK_MODE_F64 else 2e-6), (d, with_lm, mode)


def test_zero_momenta_shortcut(gb, ctx):
    """Diffeos.cxx:611-613 and :683-684: |p0| < 1e-20 gives a constant trajectory, zero momenta."""
    from deformetrica_code_gb300.deformation import Deformation
    cp, _, lm0 = small_problem(3)
    mom = np.full(cp.shape, 1e-23)
    ctx.set_mode(gb.GBK_MODE_F32C)
    df = Deformation(3, 0.3, 4, context=ctx)
    pos, mo = df.shoot(cp, mom)
    assert np.array_equal(pos, np.broadcast_to(cp, pos.shape))
    assert np.array_equal(mo[0], mom) and np.all(mo[1:] == 0)
    lm = df.flow(pos, mo, lm0)
    assert np.array_equal(lm, np.broadcast_to(lm0, lm.shape))


def test_gpu_shooting_reproduces_reference_parallel_transport(gb, ctx, K):
    """tests/unit_tests/parallel-transport (TestParallelTransport.cxx:19-85): the trajectory shot
    on the GPU (2-D, sigma 15, 30 time points) transported by the restated ParallelTransport must
    match the reference's GroundTruthMom.txt within the reference test's 1e-4 (FP64 mode).
    The transport is ill-conditioned in its input trajectory (a dense solve with cond(K) ~ 2.4e3
    and finite differences with eps = dt): relative noise of 6e-8 on the trajectory moves its
    output by ~1e-2, so the FP32 trajectory is held to 1e-3."""
    import os
    from oracle import deformation as D
    from deformetrica_code_gb300.deformation import Deformation
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "parallel_transport.npz"))
    for mode, tol in ((gb.GBK_MODE_F64, 1e-4), (gb.GBK_MODE_F32C, 1e-3)):
        ctx.set_mode(mode)
        df = Deformation(2, 15.0, 30, context=ctx)
        pos, mo = df.shoot(g["cp_regression"], g["mom_regression"])
        out = D.parallel_transport(K, 15.0, list(pos), list(mo), g["mom_transport"], g["cp_transport"],
                                   0.0, [i / 9 for i in range(10)])
        assert np.abs(out[-1] - g["ground_truth_mom"]).max() <= tol


def _meshes():
    from deformetrica_code_gb300 import meshes as M
    tp, tf = M.icosphere(2, 0.35)
    gp = M.sine_bump(tp, tf, 0.05)
    tp2, tf2 = M.icosphere(3, 0.33)
    return tp, tf, gp, tf, tp2, tf2


@pytest.mark.parametrize("kind", ["currents", "varifold"])
def test_surface_terms_match_oracle(gb, ctx, K, kind):
    from oracle import geometry as G
    from deformetrica_code_gb300.deformation import currents_match, varifold_match
    tp, tf, gp, gf, tp2, tf2 = _meshes()
    fm = currents_match if kind == "currents" else varifold_match
    om = G.currents_match if kind == "currents" else G.varifold_match
    og = G.currents_match_gradient if kind == "currents" else G.varifold_match_gradient
    for (ps, fs, pt, ft) in [(tp, tf, gp, gf), (tp, tf, tp2, tf2)]:
        rm, rg = om(K, 0.1, ps, fs, pt, ft), og(K, 0.1, ps, fs, pt, ft)
        for mode, tol in modes(gb):
            ctx.set_mode(mode)
            m, g = fm(ps, fs, pt, ft, 0.1, context=ctx)
            scale = G.currents_norm(K, 0.1, *G.centers_normals(ps, fs)) if kind == "currents" else \
                G.varifold_norm(K, 0.1, *G.varifold_normals(ps, fs))
            assert abs(m - rm) <= (1e-10 if mode == gb.GBK_MODE_F64 else 1e-5) * scale
            assert normwise_rel(g, rg) <= tol


@pytest.mark.parametrize("kind", ["currents", "varifold"])
def test_registration_step_matches_oracle_and_graph_replay(gb, ctx, K, kind):
    from oracle import deformation as D
    from deformetrica_code_gb300.deformation import Registration
    tp, tf, gp, gf, _, _ = _meshes()
    cp = grid_cp(3, 0.25, 0.75)
    mom = 0.01 * np.random.default_rng(2).standard_normal(cp.shape)
    args = dict(T=6, sigma_def=0.25, sigma_data=0.15, data_sigma2=0.01)
    L, gcp_r, gmom_r, _ = D.registration(K, cp, mom, tp, tf, gp, gf, args["T"], args["sigma_def"],
                                         args["sigma_data"], args["data_sigma2"], kind=kind)
    for mode, tol in modes(gb):
        ctx.set_mode(mode)
        reg = Registration(cp.shape[0], tp, tf, gp, gf, kind=kind, context=ctx, **args)
        outs = [reg.step(cp, mom) for _ in range(3)]  # eager, capture + replay, replay
        assert reg.graph_launches() > 20
        for ll, gc, gm in outs[1:]:  # the graph replays the eager kernels exactly
            assert np.array_equal(ll, outs[0][0]) and np.array_equal(gc, outs[0][1]) and np.array_equal(gm, outs[0][2])
        ll, gc, gm = outs[0]
        assert abs(ll[0] - L) <= (1e-9 if mode == gb.GBK_MODE_F64 else 1e-5) * abs(L)
        assert normwise_rel(gm, gmom_r) <= tol
        assert normwise_rel(gc, gcp_r) <= tol
        reg.close()


def test_pipelined_registration_equals_serial(gb, ctx, monkeypatch):
    """The default two-stream iteration (flow and control-point adjoint on a helper stream, one step
    behind) gives the one-stream iteration's loglik and gradients bit for bit, eager and replayed."""
    from deformetrica_code_gb300.deformation import Registration
    tp, tf, gp, gf, _, _ = _meshes()
    cp = grid_cp(3, 0.25, 0.75)
    mom = 0.01 * np.random.default_rng(5).standard_normal(cp.shape)
    args = dict(T=6, sigma_def=0.25, sigma_data=0.15, data_sigma2=0.01)
    for mode, _ in modes(gb):
        ctx.set_mode(mode)
        res = {}
        for pipe in ("1", "0"):
            monkeypatch.setenv("GBK_PIPELINE", pipe)
            reg = Registration(cp.shape[0], tp, tf, gp, gf, context=ctx, **args)
            res[pipe] = [reg.step(cp, mom) for _ in range(3)]  # eager, capture + replay, replay
            tr = reg.trajectories()
            res[pipe].append([tr[k] for k in ("pos", "mom", "lm", "theta", "xi_pos", "xi_mom")])
            reg.close()
        for a, b in zip(res["1"], res["0"]):
            for x, y in zip(a, b):
                assert np.array_equal(np.asarray(x), np.asarray(y))


@pytest.mark.parametrize("kind", ["currents", "varifold"])
def test_batched_atlas_matches_per_subject_oracle(gb, ctx, K, kind):
    """One batched atlas iteration over subjects with uneven target meshes equals the sum of the
    per-subject oracle registrations (DeterministicAtlas / AbstractAtlas restated), and graph replay
    reproduces the eager iteration bitwise."""
    from oracle import deformation as D
    from deformetrica_code_gb300 import meshes as M
    from deformetrica_code_gb300.deformation import Atlas
    tp, tf = M.icosphere(2, 0.35)
    targets = [M.perturbed_sphere(n, noise=0.02, seed=40 + i, radius=0.36) for i, n in enumerate((150, 420, 260))]
    cp = grid_cp(3, 0.25, 0.75)
    rng = np.random.default_rng(4)
    mom = 0.01 * rng.standard_normal((len(targets), cp.shape[0], 3))
    kw = dict(T=5, sigma_def=0.25, sigma_data=0.15, data_sigma2=0.01)
    Ls, gcp, gt = [], np.zeros_like(cp), np.zeros_like(tp)
    gms = []
    for s, (p_t, f_t) in enumerate(targets):
        L, gc, gm, info = D.registration(K, cp, mom[s], tp, tf, p_t, f_t, kw["T"], kw["sigma_def"],
                                         kw["sigma_data"], kw["data_sigma2"], kind=kind)
        Ls.append(L)
        gcp += gc
        gms.append(gm)
        gt -= info["theta"][0]
    for mode, tol in modes(gb):
        ctx.set_mode(mode)
        atlas = Atlas(cp, tp, tf, targets, kind=kind, context=ctx, **kw)
        outs = [atlas.step(mom) for _ in range(3)]  # eager, capture + replay, replay
        assert atlas.graph_launches() > 10
        for o in outs[1:]:
            for a_, b_ in zip(o, outs[0]):
                assert np.array_equal(a_, b_)
        ll, gm, gc, gtt = outs[0]
        ltol = 1e-9 if mode == gb.GBK_MODE_F64 else 1e-5
        assert abs(ll[0] - sum(Ls)) <= ltol * abs(sum(Ls))
        for s in range(len(targets)):
            assert abs(ll[3 + s] - Ls[s]) <= ltol * abs(Ls[s])
            assert normwise_rel(gm[s], gms[s]) <= tol
        assert normwise_rel(gc, gcp) <= tol
        assert normwise_rel(gtt, gt) <= tol
        atlas.close()
