"""Benchmark of the Gaussian kernel-sum hot path on one GB300 (or N replicas under torchrun).

Workload (default): forward + full adjoint of a Gaussian kernel sum at N = M = 1e6, d = 3
(the large kernel-sum sweep's biggest size): points from a mixture of 8 Gaussians (std 0.05,
means ~ U[0.15, 0.85]^3, clipped to [0,1]), weights and adjoint seeds ~ N(0,1), sigma = 0.1,
seed 3. One step = gbk_forward_adjoint: the target-side pass (Convolve + alpha-gradient, fused)
and the source-side pass (dL/dy, dL/dw, fused), every pair's distance and exp recomputed.
Metric: kernel pairs per second, pairs = N * M per step (each evaluated in both passes). The
library's default order sorts both point sets spatially and skips source chunks whose kernel
values are exactly zero; the line reports how many pairs were evaluated, and the roofline counts
evaluated pairs only.

Prints ONE JSON line (rank 0). `--impl reference` times the reference's CPU algorithm instead
(the FP64 oracle restating ExactKernel; oracle/_ref when it was built on this host). `--sweep`
runs the N x d x sigma sweep of the same step instead, one JSON line per case.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "kernel pairs/s fwd+adjoint"
UNIT = "pairs/s"
FLOPS_PER_PAIR_PASS = 26  # FP32 flops per pair of one fused Convolve + alpha-gradient pass (FMA = 2)
LANE_OPS_PER_PAIR_PASS = 16  # FP32 lane instructions per pair of that pass (FMA = 1)
# DRAM bytes (read + write) of one fused pass at N = M = 1e6, d = 3, sigma = 0.1 (the headline kernel),
# from one ncu capture (dram__bytes_read.sum + dram__bytes_write.sum); a constant, not measured per run.
TRAFFIC_1E6 = 384661248 + 313689600
TRAFFIC_SOURCE = ("constant from one ncu capture of the fused pass at N = M = 1e6, d = 3, sigma = 0.1 "
                  "(dram__bytes_read.sum + dram__bytes_write.sum); not measured in this run")
# Algorithmic FP32 lane instructions per pair (FMA = 1) of each kernel-sum operation at d = dv = 3, in
# gbk_evaluated_pairs_by_op order: Convolve 9, fused Convolve + alpha-gradient 16, alpha-gradient 13,
# varlin 18, ConvolveGradient(X, dim) 10, ConvolveHessian(X) 36, ConvolveHessian(X, r, c) 14, the
# special Hessian 23, the fused control-point adjoint update 40. Two-float CTAs and compensation
# folds are not counted.
OP_NAMES = ("convolve", "convolve_gradient_alpha", "gradient_alpha", "gradient_varlin", "gradient_dim",
            "hessian", "hessian_rowcol", "special_hessian", "adjoint_cp")
LANE_OPS_BY_OP = (9, 16, 13, 18, 10, 36, 14, 23, 40)


def pair_work(ctx, before, after, iters: int, s_per_iter: float, sm_mhz: float = 2070.0):
    """Evaluated pairs per iteration by operation (from gbk_evaluated_pairs_by_op counts taken
    around `iters` iterations), pairs/s, and the FP32 lane fraction at the nominal SM clock."""
    per = [(b - a) / iters for a, b in zip(before, after)]
    pairs = sum(per)
    lane_ops = sum(f * p for f, p in zip(LANE_OPS_BY_OP, per))
    peak_lanes = SMS * FP32_LANES * sm_mhz * 1e6
    return {"evaluated_pairs_per_iter": pairs,
            "by_op": {n: p for n, p in zip(OP_NAMES, per) if p},
            "pairs_per_s": pairs / s_per_iter,
            "fp32_lane_frac": lane_ops / s_per_iter / peak_lanes,
            "lane_frac_basis": f"sum over ops of pairs x algorithmic lane ops (d = dv = 3 counts) / "
                               f"({SMS} SMs x {FP32_LANES} lanes x {sm_mhz:.0f} MHz)"}
SMS = 152
FP32_LANES = 128


def make_workload(n: int, m: int, d: int = 3, seed: int = 3):
    rng = np.random.default_rng(seed)
    means = rng.uniform(0.15, 0.85, size=(8, d))

    def pts(k):
        comp = rng.integers(0, 8, size=k)
        p = means[comp] + 0.05 * rng.standard_normal((k, d))
        return np.clip(p, 0.0, 1.0)

    x = pts(n)
    y = pts(m)
    w = rng.standard_normal((m, d))
    a = rng.standard_normal((n, d))
    return x, y, w, a


class ClockSampler:
    """Samples nvidia-smi clocks/throttle reasons every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.gpu = gpu_index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([s.strip() for s in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx = float(s[2])
                for nm, v in zip(names, s[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
            except Exception:
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _omp_threads(n: int | None):
    """Sets the OpenMP thread count of the oracle's C port (its loops are OpenMP); returns the old one."""
    try:
        gomp = ctypes.CDLL("libgomp.so.1")
        old = gomp.omp_get_max_threads()
        if n is not None:
            gomp.omp_set_num_threads(int(n))
        return old
    except OSError:
        return None


def cpu_baseline(sample: int, kind_pref: str = "port", single_sample: int = 8192):
    """Times the FP64 CPU implementation's forward + adjoint on a bounded sample (sample x sample
    pairs) on all host cores, and on one core (single_sample x single_sample), as the reference's
    ExactKernel runs per call."""
    import oracle
    kind = "port"
    lib = None
    if kind_pref == "reference":
        try:
            lib = oracle.load("reference")
            kind = "reference"
        except Exception:
            lib = None
    if lib is None:
        lib = oracle.load("port")
    x, y, w, a = make_workload(sample, sample, seed=33)
    t0 = time.perf_counter()
    lib.fwd_adjoint(x, y, w, 0.1, a)
    dt = time.perf_counter() - t0
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    if kind == "reference":
        cores = 1  # the reference's ExactKernel is single-threaded per call
    res = {"value": sample * sample / dt, "unit": UNIT, "cores": cores,
           "kind": "reference" if kind == "reference" else "port",
           "sample": f"fwd+adjoint of {sample}x{sample} pairs (d=3, sigma=0.1), FP64, {dt:.2f} s"}
    if kind == "port" and single_sample > 0:
        old = _omp_threads(1)
        try:
            xs, ys, ws, as_ = make_workload(single_sample, single_sample, seed=34)
            t0 = time.perf_counter()
            lib.fwd_adjoint(xs, ys, ws, 0.1, as_)
            d1 = time.perf_counter() - t0
        finally:
            _omp_threads(old)
        res["single_thread"] = {"value": single_sample * single_sample / d1, "unit": UNIT, "cores": 1,
                                "sample": f"fwd+adjoint of {single_sample}x{single_sample} pairs, FP64, {d1:.2f} s"}
    return res


def accuracy(x, y, w, a, sigma, v, gx, gy, gw, sample: int = 2048, cond_sample: int = 512, seed: int = 7):
    """Errors of the four GPU outputs against the FP64 oracle: v and gx on `sample` target rows against
    all sources, gy and gw on `sample` source rows against all targets. Per output: normwise
    max_i |err_i| / max_i |ref_i| and max abs error; on the first `cond_sample` of those rows the
    condition-aware error max |err| / sum_j (1 + a_ij) |term_j| (a_ij = |x_i - y_j|^2 / sigma^2, the
    exponent's condition number) and the plain-magnitude one, max |err| / sum_j |term_j|."""
    import oracle
    port = oracle.load("port")
    rng = np.random.default_rng(seed)
    it = np.sort(rng.choice(x.shape[0], size=min(sample, x.shape[0]), replace=False))
    jt = np.sort(rng.choice(y.shape[0], size=min(sample, y.shape[0]), replace=False))
    out = sweep_errors(port, x, y, w, a, it, jt, sigma, (v, gx, gy, gw), cond=False)
    ic = np.sort(rng.choice(it, size=min(cond_sample, len(it)), replace=False))
    jc = np.sort(rng.choice(jt, size=min(cond_sample, len(jt)), replace=False))
    cond = sweep_errors(port, x, y, w, a, ic, jc, sigma, (v, gx, gy, gw), cond=True)
    for key in out:
        out[key]["condition_aware"] = cond[key]["condition_aware"]
        out[key]["plain_magnitude"] = cond[key]["plain_magnitude"]
    out["sample"] = (f"{len(it)} targets x {y.shape[0]} sources and {len(jt)} sources x {x.shape[0]} targets "
                     f"(condition-aware: {len(ic)} + {len(jc)} of those rows) vs the FP64 oracle")
    return out


def registration_workload():
    """Shooting + adjoint registration: 1,000 control points on the cell-centred grid
    {0.05, ..., 0.95}^3, momenta ~ N(0, 0.01) read as standard deviation 0.01 (seed 2; with
    standard deviation 0.1 the explicit-Euler shooting blows up, |p_t| grows 360x and the
    reference's adjoint no longer approximates the gradient), template = icosphere of radius
    0.4 centred at (0.5, 0.5, 0.5) with 10,242 vertices / 20,480 faces, target = the same sphere
    with vertices moved 0.05 sin(4 pi x) along the normals, deformation kernel width 0.15, 11
    time points (10 Euler steps, Heun flow/adjoint), currents data term of width 0.1."""
    from deformetrica_code_gb300 import meshes as M
    g = np.arange(0.05, 1.0, 0.1)
    cp = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    mom = 0.01 * np.random.default_rng(2).standard_normal(cp.shape)
    tp, tf = M.icosphere(5, 0.4)
    gp = M.sine_bump(tp, tf, 0.05, 4.0)
    return cp, mom, tp, tf, gp, tf, dict(T=11, sigma_def=0.15, sigma_data=0.1, data_sigma2=0.01)


def registration_bench(steps: int, cpu: bool = True):
    """s/iter of one registration iteration (forward + gradient) on the GPU (graph replay) in the
    compensated-FP32 and FP64 modes, the FP64 CPU oracle, and a central finite-difference check
    of the gradient (eps = 1e-3, FP64 mode)."""
    import deformetrica_code_gb300 as g
    from deformetrica_code_gb300.deformation import Registration
    cp, mom, tp, tf, gp, gf, kw = registration_workload()
    res = {"workload": "1000 CP x 10242-vertex icosphere, T=11, sigma_def 0.15, currents sigma 0.1",
           # the iteration's streams (GBK_PIPELINE=0: one) and programmatic dependent launch (GBK_PDL=0: off)
           "streams": 1 if os.environ.get("GBK_PIPELINE", "1")[:1] == "0" else 3,
           "programmatic_launch": os.environ.get("GBK_PDL", "1")[:1] != "0"}
    for name, mode, nsteps in (("f32c", g.GBK_MODE_F32C, steps), ("f64", g.GBK_MODE_F64, max(2, steps // 4))):
        ctx = g.Context(mode=mode)
        reg = Registration(cp.shape[0], tp, tf, gp, gf, context=ctx, **kw)
        for _ in range(3):  # eager, capture, first replay
            ll, gcp, gm = reg.step(cp, mom)
        c0 = ctx.evaluated_pairs_by_op()
        ts = []
        for _ in range(nsteps):
            t0 = time.perf_counter()
            ll, gcp, gm = reg.step(cp, mom)
            ts.append(time.perf_counter() - t0)
        res[name] = {"s_per_iter": statistics.mean(ts), "loglik": float(ll[0]),
                     "kernels_per_iter": reg.graph_launches()}
        if name == "f32c":
            res[name].update(pair_work(ctx, c0, ctx.evaluated_pairs_by_op(), nsteps, statistics.mean(ts)))
        if name == "f64":
            v = np.random.default_rng(9).standard_normal(mom.shape)
            eps = 1e-3
            lp = reg.step(cp, mom + eps * v)[0][0]
            lm_ = reg.step(cp, mom - eps * v)[0][0]
            fd = (lp - lm_) / (2 * eps)
            an = float(np.sum(gm * v))
            res["fd_check"] = {"eps": eps, "fd": fd, "adjoint": an, "rel_diff": abs(fd - an) / abs(an)}
        if name == "f32c":
            g32 = gm
        else:
            res["f32c_vs_f64_grad_mom_normwise"] = float(np.linalg.norm(g32 - gm, axis=1).max()
                                                         / np.linalg.norm(gm, axis=1).max())
        reg.close()
    if cpu:
        import oracle
        from oracle import deformation as D
        K = oracle.load("port")
        t0 = time.perf_counter()
        D.registration(K, cp, mom, tp, tf, gp, gf, kw["T"], kw["sigma_def"], kw["sigma_data"],
                       kw["data_sigma2"], kind="currents")
        res["cpu_fp64_oracle"] = {"s_per_iter": time.perf_counter() - t0,
                                  "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))}
    return res


def atlas_workload(nsub: int = 64, seed: int = 4):
    """Batched atlas: 64 subjects, each a perturbed sphere (Fibonacci points, radial noise 0.02,
    convex-hull triangulation) with a vertex count drawn log-uniform in [5,000, 50,000]; shared
    10,242-vertex icosphere template; 2,000 control points = a seed-fixed random subset of the 13^3
    grid on [0,1]^3; momenta ~ N(0, 0.01) (standard deviation 0.01) per subject; 11 time points;
    deformation width 0.15, currents width 0.1 (the registration workload's)."""
    from deformetrica_code_gb300 import meshes as M
    rng = np.random.default_rng(seed)
    g = np.linspace(0.0, 1.0, 13)
    grid = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    cp = grid[np.sort(rng.choice(grid.shape[0], 2000, replace=False))]
    nvs = np.round(np.exp(rng.uniform(np.log(5000), np.log(50000), nsub))).astype(int)
    targets = [M.perturbed_sphere(int(n), noise=0.02, seed=1000 + i) for i, n in enumerate(nvs)]
    mom = 0.01 * rng.standard_normal((nsub, cp.shape[0], 3))
    tp, tf = M.icosphere(5, 0.4)
    return cp, mom, tp, tf, targets, dict(T=11, sigma_def=0.15, sigma_data=0.1, data_sigma2=0.01)


def atlas_bench(steps: int, cpu: bool = True):
    """s/iter of one batched atlas iteration (all subjects, forward + gradient, graph replay)."""
    import deformetrica_code_gb300 as g
    from deformetrica_code_gb300.deformation import Atlas
    cp, mom, tp, tf, targets, kw = atlas_workload()
    ctx = g.Context()
    atlas = Atlas(cp, tp, tf, targets, context=ctx, **kw)
    for _ in range(3):
        ll, gm, gc, gt = atlas.step(mom)
    c0 = ctx.evaluated_pairs_by_op()
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        ll, gm, gc, gt = atlas.step(mom)
        ts.append(time.perf_counter() - t0)
    nfs = [t[1].shape[0] for t in targets]
    res = {"workload": f"{len(targets)} subjects, target faces {min(nfs)}..{max(nfs)}, 10242-vertex template, "
                       f"2000 CP, T=11, currents", "f32c": {"s_per_iter": statistics.mean(ts),
                                                            "loglik": float(ll[0]),
                                                            "kernels_per_iter": atlas.graph_launches()}}
    res["f32c"].update(pair_work(ctx, c0, ctx.evaluated_pairs_by_op(), steps, statistics.mean(ts)))
    atlas.close()
    if cpu:
        import oracle
        from oracle import deformation as D
        K = oracle.load("port")
        k = int(np.argsort(nfs)[len(nfs) // 2])  # the median-size subject
        t0 = time.perf_counter()
        D.registration(K, cp, mom[k], tp, tf, targets[k][0], targets[k][1], kw["T"], kw["sigma_def"],
                       kw["sigma_data"], kw["data_sigma2"])
        one = time.perf_counter() - t0
        res["cpu_fp64_oracle"] = {"s_per_subject_median": one, "s_per_iter_extrapolated": one * len(targets),
                                  "note": "one median-size subject timed, x64 extrapolated",
                                  "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))}
    return res


def data_term_bench(steps: int, cpu: bool = True, nu: int = 500, nv: int = 200, sigma: float = 0.05):
    """Currents and varifold distance + vertex gradient between two noisy tori (R 0.5, r 0.2,
    noise 0.01, seeds 5 and 6, nu x nv grid -> 2 nu nv triangles each), sigma 0.05, FP32C with
    FP64 reductions. pairs per call = 3 F^2 (template x template, template x target, target x
    target). The CPU figure is the FP64 oracle on a 100 x 40 grid (8,000 triangles)."""
    import torch
    import deformetrica_code_gb300 as g
    from deformetrica_code_gb300.deformation import currents_match, varifold_match
    from deformetrica_code_gb300.meshes import torus
    ps, fs = torus(nu, nv, seed=5)
    pt, ft = torus(nu, nv, seed=6)
    F = fs.shape[0]
    pairs = 3.0 * F * F
    ctx = g.Context()
    res = {"workload": f"two noisy tori, {F} triangles each, sigma {sigma}: distance + gradient w.r.t. all"
                       f" {ps.shape[0]} template vertices", "pairs_per_call": pairs}
    for kind, fn in (("currents", currents_match), ("varifold", varifold_match)):
        fn(ps, fs, pt, ft, sigma, context=ctx)  # warm-up (buffers, order scratch)
        torch.cuda.synchronize()
        ts = []
        ev0 = ctx.evaluated_pairs()
        for _ in range(steps):
            t0 = time.perf_counter()
            m, _ = fn(ps, fs, pt, ft, sigma, context=ctx)  # host arrays in and out, synchronous
            ts.append(time.perf_counter() - t0)
        ev = (ctx.evaluated_pairs() - ev0) / steps
        sec = statistics.median(ts)
        res[kind] = {"s_per_call": sec, "pairs_per_s": pairs / sec, "evaluated_pairs_per_call": ev,
                     "match": m, "includes": "host->device copy of both meshes, device->host gradient"}
    # point clouds (the tori's vertices, unit weights) and volume meshes (jittered tetrahedral grids)
    from deformetrica_code_gb300.deformation import pointcloud_match, volume_match
    from deformetrica_code_gb300.meshes import tet_grid
    ng = max(4, 30 * nv // 200)
    vs, cs_v = tet_grid(ng, seed=7)
    vt, ct_v = tet_grid(ng, seed=8)
    extra = {
        "pointcloud": (lambda: pointcloud_match(ps, None, pt, None, sigma, context=ctx), ps.shape[0],
                       f"two point clouds of {ps.shape[0]} points (the tori's vertices), unit weights"),
        "volume": (lambda: volume_match(vs, cs_v, vt, ct_v, sigma, context=ctx), cs_v.shape[0],
                   f"two jittered tetrahedral grids of {cs_v.shape[0]} tetrahedra"),
    }
    for kind, (fn, n_el, what) in extra.items():
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(steps):
            t0 = time.perf_counter()
            m, _ = fn()
            ts.append(time.perf_counter() - t0)
        sec = statistics.median(ts)
        res[kind] = {"workload": what + f", sigma {sigma}", "s_per_call": sec, "pairs_per_s": 3.0 * n_el * n_el / sec,
                     "match": m, "includes": "host->device copy of both objects, device->host gradient"}
    if cpu:
        import oracle
        from oracle import geometry as G
        K = oracle.load("port")
        cs, cfs = torus(100, 40, seed=5)
        ct, cft = torus(100, 40, seed=6)
        Fc = cfs.shape[0]
        cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
        for kind in ("currents", "varifold"):
            om = G.currents_match if kind == "currents" else G.varifold_match
            og = G.currents_match_gradient if kind == "currents" else G.varifold_match_gradient
            t0 = time.perf_counter()
            om(K, sigma, cs, cfs, ct, cft)
            og(K, sigma, cs, cfs, ct, cft)
            dt = time.perf_counter() - t0
            res[kind]["cpu_oracle"] = {"s_per_call": dt, "pairs_per_s": 3.0 * Fc * Fc / dt, "triangles": Fc,
                                       "cores": cores, "kind": "port (FP64)"}
        t0 = time.perf_counter()
        G.pointcloud_match(K, sigma, cs, None, ct, None)
        G.pointcloud_match_gradient(K, sigma, cs, None, ct, None)
        dt = time.perf_counter() - t0
        res["pointcloud"]["cpu_oracle"] = {"s_per_call": dt, "pairs_per_s": 3.0 * len(cs) ** 2 / dt,
                                           "points": len(cs), "cores": cores, "kind": "port (FP64)"}
        qs, qcs = tet_grid(8, seed=7)
        qt, qct = tet_grid(8, seed=8)
        t0 = time.perf_counter()
        G.volume_match(K, sigma, qs, qcs, qt, qct)
        G.volume_match_gradient(K, sigma, qs, qcs, qt, qct)
        dt = time.perf_counter() - t0
        res["volume"]["cpu_oracle"] = {"s_per_call": dt, "pairs_per_s": 3.0 * len(qcs) ** 2 / dt,
                                       "tetrahedra": len(qcs), "cores": cores, "kind": "port (FP64)"}
    return res


def optimizer_bench(cpu: bool = True, reg_iters: int = 10):
    """The device-resident FastGradientAscent (gbk_registration_optimize): (1) the reference's
    functional test 6, amygdala landmark registration (8 control points, 75/79-vertex meshes, 10
    iterations from step 1e-7, fixture tests/golden/amygdala_registration.npz) in FP64 and FP32C
    against the FP64 oracle of the same estimation on the CPU; (2) `reg_iters` iterations on the
    1000-control-point, 10,242-vertex registration workload (FP32C), per iteration and per
    evaluation."""
    import deformetrica_code_gb300 as g
    from deformetrica_code_gb300.deformation import Registration
    fx = dict(np.load(os.path.join(ROOT, "tests", "golden", "amygdala_registration.npz")))
    res = {"amygdala": {"workload": "reference functional test 6: 8 CP, 75/79-vertex currents registration, "
                                    "sigma 10, data-sigma 0.1, T = 10, 10 FastGradientAscent iterations"}}
    for name, mode in (("f64", g.GBK_MODE_F64), ("f32c", g.GBK_MODE_F32C)):
        ctx = g.Context(mode=mode)
        reg = Registration(8, fx["tmpl_pts"], fx["tmpl_tris"], fx["tgt_pts"], fx["tgt_tris"], T=10, sigma_def=10.0,
                           sigma_data=10.0, data_sigma2=0.01, kind="currents", heun=False, context=ctx)
        reg.optimize(fx["cp0"], np.zeros_like(fx["cp0"]), 10, 1e-7)  # warm-up (graph capture)
        t0 = time.perf_counter()
        r = reg.optimize(fx["cp0"], np.zeros_like(fx["cp0"]), 10, 1e-7)
        dt = time.perf_counter() - t0
        href = fx["state_history"]
        res["amygdala"][name] = {"s_total": dt, "evaluations": r["evaluations"],
                                 "history_max_rel_err_vs_reference_state": float(
                                     np.abs(r["history"] - href).max() / np.abs(href).max()),
                                 "momenta_max_rel_err_vs_reference_state": float(
                                     np.abs(r["mom"] - fx["state_momenta"]).max() / np.abs(fx["state_momenta"]).max())}
        reg.close()
    if cpu:
        import oracle
        from oracle.optimize import fast_gradient_ascent, registration_evaluator
        K = oracle.load("port")
        ev = registration_evaluator(K, fx["tmpl_pts"], fx["tmpl_tris"], fx["tgt_pts"], fx["tgt_tris"], 10, 10.0, 10.0,
                                    0.01, "currents", heun=False)
        t0 = time.perf_counter()
        r = fast_gradient_ascent(ev, [fx["cp0"], np.zeros_like(fx["cp0"])], 1e-7, 10)
        res["amygdala"]["cpu_oracle"] = {"s_total": time.perf_counter() - t0, "evaluations": r["evaluations"],
                                         "kind": "port (FP64)"}
    cp, mom, tp, tf, gp, gf, kw = registration_workload()
    ctx = g.Context()
    reg = Registration(cp.shape[0], tp, tf, gp, gf, kind="currents", context=ctx, **kw)
    reg.optimize(cp, mom, 2, 1e-4)  # warm-up
    t0 = time.perf_counter()
    r = reg.optimize(cp, mom, reg_iters, 1e-4)
    dt = time.perf_counter() - t0
    reg.close()
    res["registration_1000cp"] = {"workload": "1000 CP x 10242-vertex icosphere, T=11, sigma_def 0.15, currents "
                                              f"sigma 0.1, {reg_iters} FastGradientAscent iterations from step 1e-4, FP32C",
                                  "s_total": dt, "s_per_iteration": dt / max(1, len(r["history"]) - 1),
                                  "evaluations": r["evaluations"], "s_per_evaluation": dt / max(1, r["evaluations"]),
                                  "loglik_first_last": [float(r["history"][0].sum()), float(r["history"][-1].sum())],
                                  "stopped": r["stopped"]}
    # the reference's functional test 8: a two-object curve atlas of three subjects
    from deformetrica_code_gb300.deformation import MultiObjectAtlas
    pb = dict(np.load(os.path.join(ROOT, "tests", "golden", "parabola_atlas.npz")))
    objs = [dict(kind="curve_currents", pts=pb[f"tmpl{i}_pts"], cells=pb[f"tmpl{i}_segs"],
                 sigma=float(pb["data_kernel_width"]), sigma2=float(pb["data_sigma2"])) for i in (1, 2)]
    subjects = [[(pb[f"subj{s}_obj{i}_pts"], pb[f"subj{s}_obj{i}_segs"]) for i in (1, 2)] for s in (1, 2, 3)]
    tmpl = np.concatenate([pb["tmpl1_pts"], pb["tmpl2_pts"]])
    mom0 = np.zeros((3,) + pb["cp0"].shape)
    hist = pb["state_history"]
    res["parabola_atlas"] = {"workload": "reference functional test 8: two OrientedPolyline objects (60 points each), "
                                         "3 subjects, 40 CP, T = 10, 10 FastGradientAscent iterations over control "
                                         "points, template and momenta, lagged template"}
    for mode, name in ((g.GBK_MODE_F64, "f64"), (g.GBK_MODE_F32C, "f32c")):
        a = MultiObjectAtlas(len(pb["cp0"]), objs, subjects, int(pb["number_of_time_points"]),
                             float(pb["kernel_width"]), heun=False, context=g.Context(mode=mode))
        a.set_template_smoothing(float(pb["smoothing_width"]))
        a.optimize(pb["cp0"], tmpl, mom0, 1, 1e-3)  # warm-up: graphs captured
        t0 = time.perf_counter()
        r = a.optimize(pb["cp0"], tmpl, mom0, int(pb["max_iterations"]), float(pb["initial_step"]))
        dt = time.perf_counter() - t0
        a.close()
        res["parabola_atlas"][name] = {"s_total": dt, "evaluations": r["evaluations"],
                                       "history_max_rel_err_vs_reference_state":
                                           float(np.abs(r["history"] - hist).max() / np.abs(hist).max())}
    if cpu:
        from oracle.optimize import LaggedTemplate, fast_gradient_ascent, multi_object_atlas_evaluator
        import oracle
        K = oracle.load("port")
        oobj = [dict(kind="curve_currents", cells=pb[f"tmpl{i}_segs"], sigma=float(pb["data_kernel_width"]),
                     sigma2=float(pb["data_sigma2"]), n=len(pb[f"tmpl{i}_pts"])) for i in (1, 2)]
        lt = LaggedTemplate(tmpl, 1)
        ev = multi_object_atlas_evaluator(K, oobj, subjects, int(pb["number_of_time_points"]), float(pb["kernel_width"]),
                                          heun=False, smoothing_width=float(pb["smoothing_width"]), lag=lt)
        t0 = time.perf_counter()
        r = fast_gradient_ascent(ev, [pb["cp0"], tmpl, mom0], float(pb["initial_step"]), int(pb["max_iterations"]),
                                 set_fixed=lt.set_fixed)
        res["parabola_atlas"]["cpu_oracle"] = {"s_total": time.perf_counter() - t0, "evaluations": r["evaluations"],
                                               "kind": "port (FP64)"}
    # the reference's functional test 7: a geodesic regression of three skull curves
    from deformetrica_code_gb300.deformation import GeodesicRegression
    rg = dict(np.load(os.path.join(ROOT, "tests", "golden", "regression_skulls.npz")))
    gobj = [dict(kind="curve_varifold", pts=rg["tmpl_pts"], cells=rg["tmpl_segs"], sigma=float(rg["data_kernel_width"]),
                 sigma2=float(rg["data_sigma2"]))]
    observations = [[(rg[f"obs{k}_pts"], rg[f"obs{k}_segs"])] for k in range(3)]
    times = [int(t) for t in rg["times"]]
    res["skull_regression"] = {"workload": "reference functional test 7: geodesic regression of a 150-point "
                                           "NonOrientedPolyline through 3 observations, 16 CP, T = 5 over [0, 5], "
                                           "10 FastGradientAscent iterations over control points, momenta and template"}
    for mode, name in ((g.GBK_MODE_F64, "f64"), (g.GBK_MODE_F32C, "f32c")):
        reg = GeodesicRegression(16, gobj, observations, times, int(rg["number_of_time_points"]),
                                 float(rg["kernel_width"]), float(rg["t0"]), float(rg["tn"]), heun=False,
                                 context=g.Context(mode=mode))
        reg.set_template_smoothing(float(rg["smoothing_width"]))
        reg.optimize(rg["cp0"], np.zeros_like(rg["cp0"]), rg["tmpl_pts"], 1, 1e-3)  # warm-up: graph captured
        t0 = time.perf_counter()
        r = reg.optimize(rg["cp0"], np.zeros_like(rg["cp0"]), rg["tmpl_pts"], int(rg["max_iterations"]),
                         float(rg["initial_step"]), tolerance=float(rg["tolerance"]))
        dt = time.perf_counter() - t0
        reg.close()
        hist = rg["state_history"]
        res["skull_regression"][name] = {"s_total": dt, "evaluations": r["evaluations"],
                                         "history_max_rel_err_vs_reference_state":
                                             float(np.abs(r["history"] - hist).max() / np.abs(hist).max())}
    if cpu:
        from oracle.optimize import regression_evaluator
        oobj = [dict(kind="curve_varifold", cells=rg["tmpl_segs"], sigma=float(rg["data_kernel_width"]),
                     sigma2=float(rg["data_sigma2"]), n=len(rg["tmpl_pts"]))]
        ev = regression_evaluator(K, oobj, observations, times, int(rg["number_of_time_points"]),
                                  float(rg["kernel_width"]), float(rg["t0"]), float(rg["tn"]), heun=False,
                                  smoothing_width=float(rg["smoothing_width"]))
        t0 = time.perf_counter()
        r = fast_gradient_ascent(ev, [rg["cp0"], np.zeros_like(rg["cp0"]), rg["tmpl_pts"]], float(rg["initial_step"]),
                                 int(rg["max_iterations"]), tolerance=float(rg["tolerance"]))
        res["skull_regression"]["cpu_oracle"] = {"s_total": time.perf_counter() - t0, "evaluations": r["evaluations"],
                                                 "kind": "port (FP64)"}
    return res


def atlas_optimizer_bench(iters: int = 3):
    """FastGradientAscent of the 64-subject atlas workload on the device (control points,
    template with gradient smoothing of width 0.15, momenta), FP32C: seconds per iteration."""
    import deformetrica_code_gb300 as g
    from deformetrica_code_gb300.deformation import Atlas
    cp, mom, tp, tf, targets, kw = atlas_workload()
    ctx = g.Context()
    atlas = Atlas(cp, tp, tf, targets, kind="currents", context=ctx, **kw)
    atlas.set_template_smoothing(kw["sigma_def"])
    atlas.optimize(cp, tp, mom, 1, 1e-4)  # warm-up: eager iteration, graph capture
    t0 = time.perf_counter()
    r = atlas.optimize(cp, tp, mom, iters, 1e-4)
    dt = time.perf_counter() - t0
    atlas.close()
    return {"workload": f"64-subject atlas, {iters} FastGradientAscent iterations over control points, template "
                        "(smoothed gradient) and momenta, FP32C", "s_total": dt,
            "s_per_iteration": dt / max(1, len(r["history"]) - 1), "evaluations": r["evaluations"],
            "s_per_evaluation": dt / max(1, r["evaluations"]),
            "loglik_first_last": [float(r["history"][0].sum()), float(r["history"][-1].sum())]}


def small_kernel_bench(n: int = 4096, sigma: float = 0.2, reps: int = 50, cpu: bool = True):
    """Convolve and ConvolveGradient(X, alpha = X) at x, y = 4096 points uniform in [0,1]^3,
    weights N(0,1), sigma 0.2 (the reference's CPU-runnable kernel case): per call through the
    Python kernel object, device arrays (kernel) and host arrays (end to end), FP32C; the FP64
    oracle on the CPU beside it."""
    import torch
    import deformetrica_code_gb300 as g
    rng = np.random.default_rng(1)
    x, y, w = rng.random((n, 3)), rng.random((n, 3)), rng.standard_normal((n, 3))
    ctx = g.Context()
    res = {"workload": f"x, y: {n} points uniform in [0,1]^3, w ~ N(0,1), sigma {sigma}; alpha = x for the gradient",
           "pairs_per_call": float(n) * n}
    dev = lambda a: torch.from_numpy(a).cuda()
    for where, args in (("device", (dev(x), dev(y), dev(w))), ("host", (x, y, w))):
        k = g.GB300ExactKernel(3, sigma, context=ctx)
        X, Y, W = args
        k.SetSources(Y)
        k.SetWeights(W)
        for name, fn in (("convolve", lambda: k.Convolve(X)), ("gradient_alpha", lambda: k.ConvolveGradient(X, X))):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                fn()
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) / reps
            res.setdefault(name, {})[where] = {"s_per_call": dt, "pairs_per_s": float(n) * n / dt}
    if cpu:
        import oracle
        port = oracle.load("port")
        for name, fn in (("convolve", lambda: port.convolve(x, y, w, sigma)),
                         ("gradient_alpha", lambda: port.grad_alpha(x, y, w, sigma, x))):
            t0 = time.perf_counter()
            for _ in range(5):
                fn()
            dt = (time.perf_counter() - t0) / 5
            res[name]["cpu_oracle"] = {"s_per_call": dt, "pairs_per_s": float(n) * n / dt, "kind": "port (FP64)",
                                       "cores": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))}
    return res


def p3m_grid_size(lo, hi, sigma: float, ratio: float, padding: float = 3.0):
    """Points per axis of the particle-mesh grid (P3MKernel::DetermineGrids): the padded domain
    length over the spacing, truncated, rounded up to a power of two."""
    out = []
    for l, h in zip(lo, hi):
        n = max(int((h - l + 2 * padding * sigma) / (ratio * sigma)), 1)
        out.append(1 << (n - 1).bit_length())
    return out


def p3m_bench(reps: int = 5, cpu: bool = True, n: int = 1_000_000, sigma: float = 0.1, n_check: int = 4096,
              n_cpu: int = 20_000, spacing_ratio: float = 0.2):
    """The particle-mesh kernel (the reference's P3MKernel: grid spacing 0.2 sigma, padding 3 sigma)
    on the headline workload: N = M = 1e6 points of the 8-Gaussian mixture, sigma 0.1, Convolve
    and ConvolveGradient(X, alpha) from device arrays, timed per call with FP32 grids (f32c, the
    default context mode) and FP64 grids (f64); relative L2 errors against the exact FP64 sum on
    the first n_check targets; the FP64 numpy restatement timed on
    n_cpu targets and sources on the same grid (a bounded CPU sample: the FFTs are the same size,
    the splat and interpolation loops scale with the points)."""
    import torch
    import deformetrica_code_gb300 as g
    x, y, w, a = make_workload(n, n)
    lo, hi = np.minimum(x.min(0), y.min(0)), np.maximum(x.max(0), y.max(0))
    dom = (lo, hi)
    ctx, ctx64 = g.Context(), g.Context(mode=g.GBK_MODE_F64)
    X, Y, W, A = (torch.from_numpy(v).cuda() for v in (x, y, w, a))
    res = {"workload": f"N = M = {n}, d = 3, 8-Gaussian mixture in [0,1]^3, sigma {sigma}, spacing 0.2 sigma, "
                       "padding 3 sigma, cuFFT; grids FP32 (f32c) or FP64 (f64)",
           "grid": None, "convolve": {}, "gradient_alpha": {}}
    # exact FP64 sums on a subsample of targets
    k = g.GB300ExactKernel(3, sigma, context=ctx64)
    k.SetSources(Y)
    k.SetWeights(W)
    Xs, As = X[:n_check].contiguous(), A[:n_check].contiguous()
    exact = {"convolve": k.Convolve(Xs).cpu().numpy(), "gradient_alpha": k.ConvolveGradient(Xs, As).cpu().numpy()}
    for mode, c in (("f32c", ctx), ("f64", ctx64)):
        calls = (("convolve", lambda: g.p3m_convolve(X, Y, W, sigma, domain=dom, spacing_ratio=spacing_ratio,
                                                     context=c)),
                 ("gradient_alpha", lambda: g.p3m_convolve_gradient_alpha(X, Y, W, sigma, A, domain=dom,
                                                                          spacing_ratio=spacing_ratio, context=c)))
        for name, fn in calls:
            for _ in range(3):
                out = fn()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(reps):
                fn()
            torch.cuda.synchronize()
            dt = (time.perf_counter() - t0) / reps
            e = exact[name]
            err = float(np.linalg.norm(out[:n_check].cpu().numpy() - e) / np.linalg.norm(e))
            res[name][mode] = {"s_per_call": dt, "pairs_per_s_equivalent": float(n) * n / dt,
                               "rel_l2_err_vs_exact": err}
    res["err_sample"] = f"first {n_check} targets vs the exact FP64 GPU sum over all {n} sources"
    # ConvolveHessian(X): dv x d(d+1)/2 = 18 images, FP32 grids (timing only)
    fn = lambda: g.p3m_convolve_hessian(X, Y, W, sigma, domain=dom, spacing_ratio=spacing_ratio, context=ctx)
    for _ in range(2):
        fn()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        fn()
    torch.cuda.synchronize()
    res["hessian"] = {"f32c": {"s_per_call": (time.perf_counter() - t0) / reps, "images": 3 * 6}}
    res["grid"] = p3m_grid_size(lo, hi, sigma, spacing_ratio)
    res["spacing_ratio"] = spacing_ratio
    if cpu:
        from oracle import p3m as p3m_oracle
        xs, ys, ws, as_ = x[:n_cpu], y[:n_cpu], w[:n_cpu], a[:n_cpu]
        for name, fn in (("convolve", lambda: p3m_oracle.convolve(xs, ys, ws, sigma, lo, hi, spacing_ratio)),
                         ("gradient_alpha", lambda: p3m_oracle.convolve_gradient_alpha(xs, ys, ws, sigma, as_, lo, hi,
                                                                                       spacing_ratio))):
            t0 = time.perf_counter()
            fn()
            dt = time.perf_counter() - t0
            res[name]["cpu_oracle"] = {"s_per_call": dt, "sample": f"{n_cpu} targets and sources, same grid",
                                       "kind": "port (FP64 numpy)", "cores": 1}
    ctx.close()
    ctx64.close()
    return res


def image_window_pairs(cp, sigma: float, origin, spacing, size) -> float:
    """(pixel, control point) pairs of ConvolveImageFast: int(6 sigma) pixels per axis from the
    rounded index of y - 3 sigma, cropped to the image."""
    start = np.floor((np.asarray(cp) - 3 * sigma - np.asarray(origin)) / np.asarray(spacing) + 0.5).astype(np.int64)
    lo, hi = np.maximum(start, 0), np.minimum(start + int(6 * sigma), np.asarray(size))
    return float(np.prod(np.maximum(hi - lo, 0), axis=1).sum())


def image_bench(reps: int = 5, cpu: bool = True, n: int = 128, sigma: float = 4.0, T: int = 11):
    """The image-grid path: a 128^3 image (unit spacing, origin 0), 1,000 control points on the
    cell-centred 10^3 grid of spacing 12.8, momenta N(0, 1) x 0.5, sigma 4 pixels (windows of 24^3
    pixels). ConvolveImageFast (FP32C and FP64) on the image points displaced by 0.2 N(0,1) (device
    arrays), the full FP32C Convolve over the same pixels beside it, and the backward image-map flow
    with T = 11, Heun, with windowed sums (FP32C and FP64) and with full sums (FP32C). The FP64 numpy
    restatement of ConvolveImageFast runs on the same case (1 core)."""
    import torch
    import deformetrica_code_gb300 as g
    rng = np.random.default_rng(12)
    im = g.ImageGrid([0.0] * 3, [1.0] * 3, [n] * 3)
    c = (np.arange(10) + 0.5) * (n / 10)
    cp = np.stack(np.meshgrid(c, c, c, indexing="ij"), -1).reshape(-1, 3)
    mom = 0.5 * rng.standard_normal(cp.shape)
    ctx = g.Context()
    pts = im.points(context=ctx)
    x = pts + 0.2 * rng.standard_normal(pts.shape)
    X, Y, W = (torch.from_numpy(v).cuda() for v in (x, cp, mom))
    k = g.GB300ExactKernel(3, sigma, context=ctx)
    k.SetSources(Y)
    k.SetWeights(W)
    L = int(6 * sigma)
    win_pairs = image_window_pairs(cp, sigma, im.origin, im.spacing, im.size)
    res = {"workload": f"{n}^3 image, {len(cp)} control points, sigma {sigma} pixels (windows of {L}^3), "
                       f"T = {T} Heun for the flow",
           "window_pairs_per_call": win_pairs, "full_pairs_per_call": float(im.pixels) * len(cp)}

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    ctx64 = g.Context(mode=g.GBK_MODE_F64)
    k64 = g.GB300ExactKernel(3, sigma, context=ctx64)
    k64.SetSources(Y)
    k64.SetWeights(W)
    res["convolve_image_fast"] = {}
    for prec, kk in (("f32c", k), ("f64", k64)):
        dt = timed(lambda: kk.ConvolveImageFast(X, im))
        res["convolve_image_fast"][prec] = {"s_per_call": dt, "window_pairs_per_s": win_pairs / dt}
    v32, v64 = k.ConvolveImageFast(X, im).cpu().numpy(), k64.ConvolveImageFast(X, im).cpu().numpy()
    res["convolve_image_fast"]["f32c_rel_err_vs_f64"] = float(np.linalg.norm(v32 - v64) / np.linalg.norm(v64))
    dt = timed(lambda: k.Convolve(X))
    res["convolve_full"] = {"s_per_call": dt, "pairs_per_s": res["full_pairs_per_call"] / dt, "precision": "FP32C"}
    pos = np.repeat(cp[None], T, axis=0) + 0.5 * rng.standard_normal((T, len(cp), 3))
    momt = np.repeat(mom[None], T, axis=0)
    P, M = torch.from_numpy(pos).cuda(), torch.from_numpy(momt).cuda()
    for name, fast, c in (("flow_windowed_f32c", True, ctx), ("flow_windowed_f64", True, ctx64),
                          ("flow_full_sums_f32c", False, ctx)):
        dt = timed(lambda: g.flow_image_maps(P, M, sigma, im, heun=True, fast=fast, context=c))
        res[name] = {"s_per_flow": dt, "kernel_sums": 2 * (T - 1)}
    if cpu:
        from oracle import image as IM
        t0 = time.perf_counter()
        IM.convolve_image_fast(x, cp, mom, sigma, im.origin, im.spacing, im.size)
        dt = time.perf_counter() - t0
        res["convolve_image_fast"]["cpu_oracle"] = {"s_per_call": dt, "window_pairs_per_s": win_pairs / dt,
                                                    "kind": "port (FP64 numpy)", "cores": 1}
    return res


def fp64_gpu_pairs(n: int, sigma: float):
    """The same fused forward+adjoint step in the FP64 mode (plain FP64 kernel sums) at N = M = n."""
    import torch
    import deformetrica_code_gb300 as g
    x, y, w, a = make_workload(n, n, seed=5)
    ctx = g.Context(mode=g.GBK_MODE_F64)
    ctx.use_torch_stream()
    X, Y, W, A = (torch.from_numpy(t).cuda() for t in (x, y, w, a))
    outs = [torch.empty_like(X) for _ in range(4)]
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    step = lambda: ctx.check(ctx.lib.gbk_forward_adjoint(ctx.h, 3, 3, p(X), n, p(Y), p(W), n, sigma, p(A),
                                                         *[p(o) for o in outs]))
    step()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    step()
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e)
    return {"value": n * n / (ms / 1e3), "unit": UNIT, "N": n, "ms_per_step": ms}


def sweep_errors(port, x, y, w, a, it, jt, sigma, got, cond: bool = True):
    """Errors of the four forward + adjoint outputs (v, gx on target rows `it`; gy, gw on source rows
    `jt`) against the FP64 oracle: normwise max_i |err_i| / max_i |ref_i|, max abs, and (cond) the
    condition-aware error max |err| / sum_j (1 + a_ij) |term_j| (a_ij = |x_i - y_j|^2 / sigma^2, the
    exponent's condition number) with the plain-magnitude one, max |err| / sum_j |term_j|."""
    xs, ys, as_, ws = (np.ascontiguousarray(t) for t in (x[it], y[jt], a[it], w[jt]))
    v, gx, gy, gw = got
    cases = {"v": (v[it], port.convolve(xs, y, w, sigma), lambda c: port.convolve_mag(xs, y, w, sigma, c)),
             "gx": (gx[it], port.grad_alpha(xs, y, w, sigma, as_), lambda c: port.grad_alpha_mag(xs, y, w, sigma, as_, c)),
             "gy": (gy[jt], port.grad_alpha(ys, x, a, sigma, ws), lambda c: port.grad_alpha_mag(ys, x, a, sigma, ws, c)),
             "gw": (gw[jt], port.convolve(ys, x, a, sigma), lambda c: port.convolve_mag(ys, x, a, sigma, c))}
    out = {}
    for key, (g_, r, mag) in cases.items():
        e = g_ - r
        out[key] = {"normwise": float(np.linalg.norm(e, axis=1).max() / np.linalg.norm(r, axis=1).max()),
                    "max_abs": float(np.abs(e).max())}
        if cond:
            out[key]["condition_aware"] = float((np.abs(e) / np.maximum(mag(True), 1e-300)).max())
            out[key]["plain_magnitude"] = float((np.abs(e) / np.maximum(mag(False), 1e-300)).max())
    return out


def sweep_mixture(ns, ds, sigmas, fp64_max_n: int = 100_000, sample: int = 4096):
    """The large kernel-sum + adjoint sweep: fwd+adjoint at N = M for every (N, d, sigma) on the
    8-Gaussian mixture (seed 3), FP32C in the default order; FP64 mode timed too for N <= fp64_max_n.
    Errors per output against the FP64 oracle on `sample` rows against all partners. Prints one
    JSON line per case."""
    import torch
    import deformetrica_code_gb300 as g
    import oracle
    port = oracle.load("port")
    ctx = g.Context()
    ctx.use_torch_stream()
    c64 = g.Context(mode=g.GBK_MODE_F64)
    c64.use_torch_stream()
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    stream = torch.cuda.current_stream()

    def timed(c, d, n, X, Y, W, A, outs, sigma):
        step = lambda: c.check(c.lib.gbk_forward_adjoint(c.h, d, d, p(X), n, p(Y), p(W), n, sigma, p(A),
                                                         *[p(o) for o in outs]))
        step()
        torch.cuda.synchronize()
        ev0, ms, k = c.evaluated_pairs(), [], 0
        while k < 3 or (sum(ms) < 300.0 and k < 50):
            s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s_.record(stream)
            step()
            e_.record(stream)
            torch.cuda.synchronize()
            ms.append(s_.elapsed_time(e_))
            k += 1
        return statistics.median(ms), (c.evaluated_pairs() - ev0) / k

    for d in ds:
        for n in ns:
            x, y, w, a = make_workload(n, n, d=d, seed=3)
            X, Y, W, A = (torch.from_numpy(t).cuda() for t in (x, y, w, a))
            outs = [torch.empty_like(X) for _ in range(4)]
            rng = np.random.default_rng(7)
            k_rows = min(sample if n <= 100_000 else 1024, n)  # bounds the FP64 oracle's time per case
            it = np.sort(rng.choice(n, size=k_rows, replace=False))
            jt = np.sort(rng.choice(n, size=k_rows, replace=False))
            for sigma in sigmas:
                ms, ev = timed(ctx, d, n, X, Y, W, A, outs, sigma)
                got = [o.cpu().numpy() for o in outs]
                errs = sweep_errors(port, x, y, w, a, it, jt, sigma, got)
                line = {"sweep": "mixture fwd+adjoint", "N": n, "d": d, "sigma": sigma, "ms": ms,
                        "pairs_per_s": float(n) * n / (ms / 1e3), "evaluated_fraction": ev / (2.0 * n * n),
                        "errors": errs, "error_sample": f"{len(it)} rows vs all {n} partners, FP64 oracle"}
                if float(n) * n < 2.0 ** 30:  # below the size rule: every order, timed and checked
                    line["orders"] = {}
                    for name, order in (("off", g.GBK_ORDER_OFF), ("two_float", g.GBK_ORDER_TWO_FLOAT),
                                        ("spatial", g.GBK_ORDER_SPATIAL)):
                        ctx.set_order(order)
                        ms_o, ev_o = timed(ctx, d, n, X, Y, W, A, outs, sigma)
                        got_o = [o.cpu().numpy() for o in outs]
                        e_o = sweep_errors(port, x, y, w, a, it, jt, sigma, got_o, cond=False)
                        line["orders"][name] = {
                            "ms": ms_o, "evaluated_fraction": ev_o / (2.0 * n * n),
                            "worst_normwise": max(v["normwise"] for v in e_o.values())}
                    ctx.set_order(g.GBK_ORDER_AUTO)
                if n <= fp64_max_n:
                    ms64, _ = timed(c64, d, n, X, Y, W, A, [torch.empty_like(X) for _ in range(4)], sigma)
                    line["fp64_gpu"] = {"ms": ms64, "pairs_per_s": float(n) * n / (ms64 / 1e3)}
                print(json.dumps(line), flush=True)
            del X, Y, W, A, outs
            torch.cuda.empty_cache()
    return 0


def threaded_fwd_adjoint(lib, x, y, w, sigma, a, nthreads: int):
    """The reference's forward + adjoint with its four kernel calls split into blocks of target rows
    run on nthreads host threads (every output row depends on its own target row only; the calls
    release the GIL): the reference's single-threaded ExactKernel on all host cores, as its atlas
    runs one kernel object per thread."""
    from concurrent.futures import ThreadPoolExecutor

    def split(fn, X, Y, W, A=None):
        blocks = np.array_split(np.arange(X.shape[0]), nthreads)
        jobs = [(np.ascontiguousarray(X[b]), None if A is None else np.ascontiguousarray(A[b])) for b in blocks]
        with ThreadPoolExecutor(nthreads) as ex:
            outs = list(ex.map(lambda j: fn(j[0], Y, W, sigma) if j[1] is None else fn(j[0], Y, W, sigma, j[1]),
                               jobs))
        return np.concatenate(outs, axis=0)

    v = split(lib.convolve, x, y, w)
    gx = split(lib.grad_alpha, x, y, w, a)
    gw = split(lib.convolve, y, x, a)
    gy = split(lib.grad_alpha, y, x, a, w)
    return v, gx, gy, gw


def run_reference_arm(args, rank, world):
    if rank != 0:
        return 0
    sample = args.cpu_sample
    x, y, w, a = make_workload(sample, sample, seed=33)
    import oracle
    lib = oracle.load("port")
    kind = "port"
    try:
        lib = oracle.load("reference")
        kind = "reference"
    except Exception:
        pass
    nthreads = os.cpu_count() or 1
    if kind == "reference":  # single-threaded per call: row blocks on every host thread
        step = lambda xs, ys, ws, as_: threaded_fwd_adjoint(lib, xs, ys, ws, 0.1, as_, nthreads)
    else:  # the C port threads its own loops
        step = lambda xs, ys, ws, as_: lib.fwd_adjoint(xs, ys, ws, 0.1, as_)
    for _ in range(args.warmup if args.warmup < 1 else 1):
        step(x[:256], y[:256], w[:256], a[:256])
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step(x, y, w, a)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * statistics.mean(times)
    value = sample * sample / (ms / 1e3)
    cores = nthreads if kind == "reference" else int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"fwd+adjoint Gaussian kernel sum, bounded CPU sample {sample}x{sample}"
                                   f" of the N=M=1e6 d=3 mixture workload", "d": 3, "dv": 3, "sigma": 0.1},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": kind,
                             "sample": f"{sample}x{sample} pairs per step, FP64"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=1_000_000, help="targets = sources per step")
    ap.add_argument("--sigma", type=float, default=0.1)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-sample", type=int, default=65536)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--fp64-n", type=int, default=200_000)
    ap.add_argument("--no-registration", action="store_true")
    ap.add_argument("--reg-steps", type=int, default=10)
    ap.add_argument("--no-atlas", action="store_true")
    ap.add_argument("--atlas-steps", type=int, default=3)
    ap.add_argument("--sweep", action="store_true",
                    help="run the N x d x sigma sweep instead (one JSON line per case)")
    ap.add_argument("--sweep-n", default="1e4,3e4,1e5,3e5,1e6")
    ap.add_argument("--sweep-d", default="2,3")
    ap.add_argument("--sweep-sigma", default="0.02,0.1,0.5")
    ap.add_argument("--no-data-terms", action="store_true")
    ap.add_argument("--no-small", action="store_true", help="skip the 4096-point kernel-sum case")
    ap.add_argument("--no-optimizer", action="store_true", help="skip the registration optimiser runs")
    ap.add_argument("--no-p3m", action="store_true", help="skip the particle-mesh kernel case")
    ap.add_argument("--no-image", action="store_true", help="skip the image-grid case")
    ap.add_argument("--data-term-steps", type=int, default=3)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        return run_reference_arm(args, rank, world)
    if args.sweep:
        import torch
        torch.cuda.set_device(local_rank)
        ns = [int(float(v)) for v in args.sweep_n.split(",")]
        return sweep_mixture(ns, [int(v) for v in args.sweep_d.split(",")],
                             [float(v) for v in args.sweep_sigma.split(",")])

    import torch
    import deformetrica_code_gb300 as g

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    n = m = args.n
    d = dv = 3
    x, y, w, a = make_workload(n, m, seed=3 + rank)
    dev = lambda arr: torch.from_numpy(arr).cuda()
    X, Y, W, A = dev(x), dev(y), dev(w), dev(a)
    V = torch.empty((n, dv), dtype=torch.float64, device="cuda")
    GX = torch.empty((n, d), dtype=torch.float64, device="cuda")
    GY = torch.empty((m, d), dtype=torch.float64, device="cuda")
    GW = torch.empty((m, dv), dtype=torch.float64, device="cuda")
    ctx = g.Context(local_rank)
    lib = ctx.lib
    stream = torch.cuda.current_stream()
    ctx.use_torch_stream()  # the kernels and the CUDA events share torch's current stream
    p = lambda t: ctypes.c_void_p(t.data_ptr())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MiB > L2

    def step():
        ctx.check(lib.gbk_forward_adjoint(ctx.h, d, dv, p(X), n, p(Y), p(W), m, args.sigma, p(A),
                                          p(V), p(GX), p(GY), p(GW)))

    def one_side():  # the dominant kernel alone: one fused target-side pass
        ctx.check(lib.gbk_convolve_and_gradient_alpha(ctx.h, d, dv, p(X), n, p(Y), p(W), m,
                                                      args.sigma, p(A), p(V), p(GX)))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    ev0 = ctx.evaluated_pairs()

    # ---- timed region: K steps, L2 flushed between steps (outside the events) ----
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = ctx.launch_count()
    with ClockSampler(local_rank) as clk:
        for i in range(args.steps):
            flush.zero_()
            evs[i][0].record(stream)
            step()
            evs[i][1].record(stream)
        torch.cuda.synchronize()
        launches = ctx.launch_count() - l0
        ev1 = ctx.evaluated_pairs()
        step_ms = [s.elapsed_time(e) for s, e in evs]
        # dominant kernel: one fused pass, averaged over launches
        kev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(3)]
        for s, e in kev:
            flush.zero_()
            s.record(stream)
            one_side()
            e.record(stream)
        torch.cuda.synchronize()
    launch_cfg = ctx.last_launch()  # the fused pass's compiled variant and source splits
    ev_pass = (ctx.evaluated_pairs() - ev1) / len(kev)  # pairs one fused pass evaluated
    ev_step = (ev1 - ev0) / args.steps  # both passes of a step
    kernel_ms = statistics.mean(s.elapsed_time(e) for s, e in kev)
    ms = sum(step_ms) / len(step_ms)
    if dist:
        from deformetrica_code_gb300.distributed import max_over_ranks
        ms = max_over_ranks(ms)
        dist.barrier()

    pairs = float(n) * m
    value = pairs * world / (ms / 1e3)

    # ---- end to end through the public API with pinned host buffers ----
    pin = lambda arr: torch.from_numpy(arr).pin_memory()
    hx, hy, hw, ha = pin(x), pin(y), pin(w), pin(a)
    hv = torch.empty((n, dv), dtype=torch.float64).pin_memory()
    hgx = torch.empty((n, d), dtype=torch.float64).pin_memory()
    hgy = torch.empty((m, d), dtype=torch.float64).pin_memory()
    hgw = torch.empty((m, dv), dtype=torch.float64).pin_memory()

    def e2e_step():
        ctx.check(lib.gbk_forward_adjoint(ctx.h, d, dv, p(hx), n, p(hy), p(hw), m, args.sigma, p(ha),
                                          p(hv), p(hgx), p(hgy), p(hgw)))

    if args.e2e_steps > 0:
        e2e_step()
    e2e_t = [float("nan")]
    if args.e2e_steps > 0:
        e2e_t = []
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        e2e_step()  # synchronous: returns with results in host memory
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = statistics.mean(e2e_t)
    h2d = 8 * (n * d + m * d + m * dv + n * dv)
    d2h = 8 * (n * dv + n * d + m * d + m * dv)

    clocks = clk.summary()
    sm_mhz = clocks["sm_mhz"] or 2070.0
    peak_tflops = SMS * FP32_LANES * 2 * sm_mhz * 1e6 / 1e12
    achieved = FLOPS_PER_PAIR_PASS * ev_pass / (kernel_ms / 1e3) / 1e12  # evaluated pairs only

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32c", "data": "synthetic",
            "config": {"workload": f"fwd+adjoint Gaussian kernel sum N=M={n} d=3 dv=3 sigma={args.sigma}"
                                   " (8-Gaussian mixture, std 0.05, seed 3)",
                       "N": n, "M": m, "d": d, "dv": dv, "sigma": args.sigma,
                       "pairs_per_step": pairs, "l2": "flushed between steps (256 MiB write)",
                       "order": "GBK_ORDER_AUTO: Morton-sorted targets and sources, source chunks whose"
                                " kernel values are exactly zero skipped",
                       "evaluated_pairs_per_step": ev_step, "evaluated_fraction": ev_step / (2.0 * pairs),
                       "parallelism": f"replicas{world}"},
            "gpu_launches": launches,
            "e2e": {"value": pairs * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "s_per_step": e2e_s},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_tflops, "unit": "TFLOP/s",
                         "frac": achieved / peak_tflops,
                         "traffic": TRAFFIC_1E6 if n == 1_000_000 else None,
                         "traffic_source": TRAFFIC_SOURCE,
                         "kernel": "pair_kernel<OpConvGradAlpha<3,3,true>, float2 lanes, bulk-staged source tiles>"
                                   " (one fused pass)",
                         "launch_config": {"variant": launch_cfg[0], "nsplit": launch_cfg[1]},
                         "fp32_lane_frac": LANE_OPS_PER_PAIR_PASS * ev_pass / (kernel_ms / 1e3)
                         / (SMS * FP32_LANES * sm_mhz * 1e6),
                         "evaluated_pairs_per_pass": ev_pass,
                         "kernel_ms": kernel_ms,
                         "peak_source": f"nominal FP32 {SMS} SMs x {FP32_LANES} lanes x 2 flops x median sampled SM clock {sm_mhz:.0f} MHz"},
            "clocks": clocks,
        }
        if not args.no_accuracy:
            line["accuracy"] = accuracy(x, y, w, a, args.sigma, V.cpu().numpy(), GX.cpu().numpy(),
                                        GY.cpu().numpy(), GW.cpu().numpy())
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(args.cpu_sample)
        if not args.no_fp64:
            line["fp64_gpu"] = fp64_gpu_pairs(args.fp64_n, args.sigma)
        if not args.no_registration:
            line["shooting_adjoint"] = registration_bench(args.reg_steps, cpu=not args.no_cpu_baseline)
        if not args.no_atlas:
            line["atlas"] = atlas_bench(args.atlas_steps, cpu=not args.no_cpu_baseline)
        if not args.no_data_terms:
            line["data_terms"] = data_term_bench(args.data_term_steps, cpu=not args.no_cpu_baseline)
        if not args.no_small:
            line["small_kernel_sum"] = small_kernel_bench(cpu=not args.no_cpu_baseline)
        if not args.no_p3m:
            line["p3m"] = p3m_bench(cpu=not args.no_cpu_baseline)
        if not args.no_image:
            line["image_grid"] = image_bench(cpu=not args.no_cpu_baseline)
        if not args.no_optimizer:
            line["optimizer"] = optimizer_bench(cpu=not args.no_cpu_baseline)
            if not args.no_atlas:
                line["optimizer"]["atlas_64_subjects"] = atlas_optimizer_bench()
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
