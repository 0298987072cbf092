"""Python interface to the device-resident deformation engine, data terms and registration step.

Mirrors the reference's Diffeos (Diffeos.cxx:589-712), AdjointEquationsIntegrator
(AdjointEquationsIntegrator.cxx:33-570), the surface data terms (OrientedSurfaceMesh.cxx,
NonOrientedSurfaceMesh.cxx) and one DeterministicAtlas subject iteration
(DeterministicAtlas.cxx:99-280, AbstractAtlas.cxx:559-613). Inputs are float64 numpy arrays
(host) or CUDA float64 torch tensors; every computation runs in libgbkernel.so.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .kernel import Context, _empty_like, _is_torch, _ptr


def _f64(a):
    if _is_torch(a):
        return a.contiguous()
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a):
    if _is_torch(a):
        import torch
        return a.to(torch.int32).contiguous()
    return np.ascontiguousarray(a, dtype=np.int32)


class Deformation:
    """Landmark diffeomorphism: Gaussian kernel of width sigma, T time points on [0, 1]."""

    def __init__(self, d: int, sigma: float, T: int, heun: bool = True, context: Context | None = None):
        self.d, self.sigma, self.T, self.heun = d, float(sigma), int(T), bool(heun)
        self.ctx = context or Context()

    def _call(self, name, *args, arrays=()):
        self.ctx.bind_stream(*arrays)
        self.ctx.check(getattr(self.ctx.lib, name)(self.ctx.h, *args))

    def shoot(self, cp0, mom0):
        cp0, mom0 = _f64(cp0), _f64(mom0)
        n = cp0.shape[0]
        pos = _empty_like(cp0, (self.T, n, self.d))
        mom = _empty_like(cp0, (self.T, n, self.d))
        self._call("gbk_shoot", self.d, n, _ptr(cp0), _ptr(mom0), self.T, self.sigma, _ptr(pos),
                   _ptr(mom), arrays=(cp0, mom0))
        return pos, mom

    def flow(self, pos, mom, lm0):
        pos, mom, lm0 = _f64(pos), _f64(mom), _f64(lm0)
        lm = _empty_like(lm0, (self.T, lm0.shape[0], self.d))
        self._call("gbk_flow_landmarks", self.d, pos.shape[1], _ptr(pos), _ptr(mom), self.T, self.sigma,
                   lm0.shape[0], _ptr(lm0), int(self.heun), _ptr(lm), arrays=(pos, mom, lm0))
        return lm

    def adjoint_landmarks(self, pos, mom, lm, theta_final):
        pos, mom, lm, th = _f64(pos), _f64(mom), _f64(lm), _f64(theta_final)
        theta = _empty_like(th, (self.T, lm.shape[1], self.d))
        self._call("gbk_adjoint_landmarks", self.d, pos.shape[1], _ptr(pos), _ptr(mom), self.T, self.sigma,
                   lm.shape[1], _ptr(lm), _ptr(th), int(self.heun), _ptr(theta), arrays=(pos, mom, lm, th))
        return theta

    def compute_update_at(self, pos, mom, xi_pos, xi_mom, lm=None, theta=None):
        pos, mom, xp, xm = (_f64(a) for a in (pos, mom, xi_pos, xi_mom))
        nlm = 0 if lm is None else lm.shape[0]
        lm = None if lm is None else _f64(lm)
        theta = None if theta is None else _f64(theta)
        dpos = _empty_like(pos, pos.shape)
        dmom = _empty_like(pos, pos.shape)
        self._call("gbk_compute_update_at", self.d, pos.shape[0], _ptr(pos), _ptr(mom), _ptr(xp), _ptr(xm),
                   nlm, _ptr(lm), _ptr(theta), self.sigma, _ptr(dpos), _ptr(dmom), arrays=(pos, mom, xp, xm))
        return dpos, dmom

    def adjoint_diffeo(self, pos, mom, lm=None, theta=None):
        pos, mom = _f64(pos), _f64(mom)
        nlm = 0 if lm is None else lm.shape[1]
        lm = None if lm is None else _f64(lm)
        theta = None if theta is None else _f64(theta)
        xp = _empty_like(pos, pos.shape)
        xm = _empty_like(pos, pos.shape)
        self._call("gbk_adjoint_diffeo", self.d, pos.shape[1], _ptr(pos), _ptr(mom), self.T, self.sigma, nlm,
                   _ptr(lm), _ptr(theta), int(self.heun), _ptr(xp), _ptr(xm), arrays=(pos, mom))
        return xp, xm


def _surface(name, ctx, pts, tris, pts_t, tris_t, sigma, grad=True, with_dim=False):
    ctx = ctx or Context()
    pts, pts_t = _f64(pts), _f64(pts_t)
    tris, tris_t = _i32(tris), _i32(tris_t)
    match = np.zeros(1)
    g = np.zeros(pts.shape) if grad else None
    ctx.bind_stream()
    dim = (pts.shape[1],) if with_dim else ()
    ctx.check(getattr(ctx.lib, name)(ctx.h, *dim, pts.shape[0], _ptr(pts), tris.shape[0], _ptr(tris),
                                     pts_t.shape[0], _ptr(pts_t), tris_t.shape[0], _ptr(tris_t),
                                     float(sigma), ctypes.c_void_p(match.ctypes.data), _ptr(g)))
    return float(match[0]), g


def currents_match(pts, tris, pts_t, tris_t, sigma, grad=True, context: Context | None = None):
    """Currents distance |S - T|^2 and its gradient w.r.t. pts (OrientedSurfaceMesh.cxx:124-241)."""
    return _surface("gbk_currents_match", context, pts, tris, pts_t, tris_t, sigma, grad)


def varifold_match(pts, tris, pts_t, tris_t, sigma, grad=True, context: Context | None = None):
    """Varifold distance and its gradient w.r.t. pts (NonOrientedSurfaceMesh.cxx:124-265)."""
    return _surface("gbk_varifold_match", context, pts, tris, pts_t, tris_t, sigma, grad)


def curve_currents_match(pts, segs, pts_t, segs_t, sigma, grad=True, context: Context | None = None):
    """Currents distance between polylines of 2-point segments (d = 2 or 3) and its gradient w.r.t.
    pts (OrientedPolyLine::ComputeMatch, ComputeMatchGradient)."""
    return _surface("gbk_curve_currents_match", context, pts, segs, pts_t, segs_t, sigma, grad, True)


def curve_varifold_match(pts, segs, pts_t, segs_t, sigma, grad=True, context: Context | None = None):
    """Varifold distance between polylines and its gradient w.r.t. pts
    (NonOrientedPolyLine.cxx:125-256)."""
    return _surface("gbk_curve_varifold_match", context, pts, segs, pts_t, segs_t, sigma, grad, True)


def pointcloud_match(pts, w, pts_t, w_t, sigma, grad=True, context: Context | None = None):
    """Weighted point-cloud distance and its gradient w.r.t. pts (PointCloud.cxx:104-198); w, w_t
    are per-point weights (None: unit weights). The gradient follows the context's gradient mode."""
    ctx = context or Context()
    pts, pts_t = _f64(pts), _f64(pts_t)
    w = None if w is None else _f64(w)
    w_t = None if w_t is None else _f64(w_t)
    if pts.shape[1] != pts_t.shape[1] or (w is not None and len(w) != len(pts)) or (
            w_t is not None and len(w_t) != len(pts_t)):
        raise ValueError("point and weight counts or dimensions disagree")
    match = np.zeros(1)
    g = np.zeros(pts.shape) if grad else None
    ctx.bind_stream()
    ctx.check(ctx.lib.gbk_pointcloud_match(ctx.h, pts.shape[1], pts.shape[0], _ptr(pts), _ptr(w), pts_t.shape[0],
                                           _ptr(pts_t), _ptr(w_t), float(sigma), ctypes.c_void_p(match.ctypes.data),
                                           _ptr(g)))
    return float(match[0]), g


def volume_match(pts, cells, pts_t, cells_t, sigma, grad=True, context: Context | None = None):
    """Oriented volume-mesh distance (tetrahedra in 3-D, triangles in 2-D) and its gradient w.r.t.
    pts (OrientedVolumeMesh.cxx:115-280). The gradient follows the context's gradient mode."""
    return _surface("gbk_volume_match", context, pts, cells, pts_t, cells_t, sigma, grad, True)


def landmark_match(pts, pts_t, grad=True, context: Context | None = None):
    """|S - T|^2 and 2 (S - T) over corresponding points (Landmark.cxx:288-322)."""
    ctx = context or Context()
    pts, pts_t = _f64(pts), _f64(pts_t)
    if tuple(pts.shape) != tuple(pts_t.shape):
        raise ValueError("landmark objects need the same number of points")
    match = np.zeros(1)
    g = np.zeros(pts.shape) if grad else None
    ctx.bind_stream()
    ctx.check(ctx.lib.gbk_landmark_match(ctx.h, pts.shape[1], pts.shape[0], _ptr(pts), _ptr(pts_t),
                                         ctypes.c_void_p(match.ctypes.data), _ptr(g)))
    return float(match[0]), g


class Registration:
    """One subject of DeterministicAtlas with a frozen template, replayed from a CUDA graph: a
    triangle mesh in 3-D (kind "currents" / "varifold"), a polyline of 2-point segments in 2-D or
    3-D ("curve_currents" / "curve_varifold"), a weighted point cloud ("pointcloud": cells are
    ignored, weights by `tmpl_weights` / `tgt_weights`), a volume mesh of (d + 1)-vertex cells
    ("volume") or landmarks ("landmark"); the dimension is the template's."""

    KINDS = {"currents": 0, "varifold": 1, "curve_currents": 2, "curve_varifold": 3, "pointcloud": 4, "volume": 5,
             "landmark": 6}

    def __init__(self, ncp: int, tmpl_pts, tmpl_tris, tgt_pts, tgt_tris, T: int, sigma_def: float,
                 sigma_data: float, data_sigma2: float, kind: str = "currents", heun: bool = True,
                 context: Context | None = None, tmpl_weights=None, tgt_weights=None):
        self.ctx = context or Context()
        self.ncp, self.T = int(ncp), int(T)
        tp, gp = _f64(tmpl_pts), _f64(tgt_pts)
        pointwise = kind in ("pointcloud", "landmark")
        tt = _i32(np.zeros((tp.shape[0], 1)) if pointwise else tmpl_tris)
        gt = _i32(np.zeros((gp.shape[0], 1)) if pointwise else tgt_tris)
        self.nv, self.d, self.nv_t = tp.shape[0], tp.shape[1], gp.shape[0]
        if kind == "landmark" and gp.shape != tp.shape:
            raise ValueError("landmark objects need the same number of points")
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.gbk_registration_create(
            self.ctx.h, self.d, self.ncp, tp.shape[0], _ptr(tp), tt.shape[0], _ptr(tt), gp.shape[0], _ptr(gp),
            gt.shape[0], _ptr(gt), self.T, float(sigma_def), float(sigma_data), float(data_sigma2),
            self.KINDS[kind], int(heun), ctypes.byref(h)))
        self.h = h
        if tmpl_weights is not None or tgt_weights is not None:
            self.set_point_weights(tmpl_weights, tgt_weights)

    @classmethod
    def from_objects(cls, ncp: int, objects, targets, T: int, sigma_def: float, heun: bool = True,
                     context: Context | None = None):
        """A registration whose template has several objects (gbk_registration_create_multi):
        `objects` as for MultiObjectAtlas, `targets` one (points, cells) per object. Point weights of
        point-cloud objects go through set_point_weights over all template / target points."""
        self = cls.__new__(cls)
        self.ctx = context or Context()
        self.ncp, self.T = int(ncp), int(T)
        d = int(np.asarray(objects[0]["pts"]).shape[1])
        kinds, nv, pts, nc, cells = _objects_arrays(objects, d, cls.KINDS)
        objs_t = [dict(o, pts=t[0], cells=t[1]) for o, t in zip(objects, targets)]
        _, nv_t, pts_t, nc_t, cells_t = _objects_arrays(objs_t, d, cls.KINDS)
        sd = np.array([float(o["sigma"]) for o in objects])
        s2 = np.array([float(o["sigma2"]) for o in objects])
        self.nv, self.d, self.nv_t = int(nv.sum()), d, int(nv_t.sum())
        c = lambda a: ctypes.c_void_p(a.ctypes.data)
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.gbk_registration_create_multi(
            self.ctx.h, d, self.ncp, len(objects), c(kinds), c(nv), c(pts), c(nc), c(cells), c(nv_t), c(pts_t), c(nc_t),
            c(cells_t), c(sd), c(s2), self.T, float(sigma_def), int(heun), ctypes.byref(h)))
        self.h = h
        return self

    def set_template(self, pts):
        """Replaces the template points (all objects)."""
        pts = _f64(pts)
        if tuple(pts.shape) != (self.nv, self.d):
            raise ValueError("template shape")
        self.ctx.check(self.ctx.lib.gbk_registration_set_template(self.h, _ptr(pts)))

    def set_point_weights(self, tmpl_weights=None, tgt_weights=None):
        """Point weights of a point-cloud registration (None keeps the current ones)."""
        w = None if tmpl_weights is None else _f64(tmpl_weights)
        wt = None if tgt_weights is None else _f64(tgt_weights)
        if (w is not None and len(w) != self.nv) or (wt is not None and len(wt) != self.nv_t):
            raise ValueError("one weight per point")
        self.ctx.check(self.ctx.lib.gbk_registration_set_point_weights(self.h, _ptr(w), _ptr(wt)))

    def set_graph(self, enable: bool):
        self.ctx.check(self.ctx.lib.gbk_registration_set_graph(self.h, int(enable)))

    def step(self, cp, mom):
        """Returns (loglik[5] = L, L_data, L_reg, match, <Kp,p>), dL/dcp, dL/dp."""
        cp, mom = _f64(cp), _f64(mom)
        if tuple(cp.shape) != (self.ncp, self.d) or tuple(mom.shape) != (self.ncp, self.d):
            raise ValueError(f"expected control points and momenta of shape {(self.ncp, self.d)}")
        ll = np.zeros(5)
        gcp = _empty_like(cp, cp.shape)
        gmom = _empty_like(cp, cp.shape)
        self.ctx.check(self.ctx.lib.gbk_registration_step(self.h, _ptr(cp), _ptr(mom),
                                                          ctypes.c_void_p(ll.ctypes.data), _ptr(gcp), _ptr(gmom)))
        return ll, gcp, gmom

    def graph_launches(self) -> int:
        return int(self.ctx.lib.gbk_registration_graph_launches(self.h))

    STOP = {0: "max_iterations", 1: "line_search", 2: "tolerance"}

    def optimize(self, cp, mom, max_iterations: int, initial_step: float = 1e-3, optimize_cp: bool = True,
                 max_line_search: int = 10, shrink: float = 0.5, expand: float = 1.2, tolerance: float = 1e-4,
                 nb_iter_freeze: int = 3):
        """The context's estimator (the reference's FastGradientAscent by default, or GradientAscent)
        over control points and momenta, on the device
        (gbk_registration_optimize). Returns a dict: cp, mom (final fixed effects), aux_cp, aux_mom,
        grad_cp, grad_mom (extrapolated point and gradient there), history ([data, regularity] per
        iteration), step, tau, freeze_counter, grad_sq_norms, evaluations, stopped."""
        cp = np.array(cp, dtype=np.float64)
        mom = np.array(mom, dtype=np.float64)
        if cp.shape != (self.ncp, self.d) or mom.shape != (self.ncp, self.d):
            raise ValueError(f"expected control points and momenta of shape {(self.ncp, self.d)}")
        hist = np.zeros((max_iterations + 1, 2))
        info = np.zeros(8)
        aux_cp, aux_mom, g_cp, g_mom = (np.zeros_like(cp) for _ in range(4))
        iters = ctypes.c_int(0)
        c = lambda a: ctypes.c_void_p(a.ctypes.data)
        self.ctx.check(self.ctx.lib.gbk_registration_optimize(
            self.h, c(cp), c(mom), int(optimize_cp), int(max_iterations), float(initial_step), int(max_line_search),
            float(shrink), float(expand), float(tolerance), int(nb_iter_freeze), c(hist), ctypes.byref(iters), c(info),
            c(aux_cp), c(aux_mom), c(g_cp), c(g_mom)))
        return {"cp": cp, "mom": mom, "aux_cp": aux_cp, "aux_mom": aux_mom, "grad_cp": g_cp, "grad_mom": g_mom,
                "history": hist[:iters.value], "step": info[:2] if optimize_cp else info[1:2], "tau": float(info[2]),
                "freeze_counter": int(info[3]), "grad_sq_norms": info[4:6] if optimize_cp else info[5:6],
                "evaluations": int(info[6]), "stopped": self.STOP[int(info[7])]}

    def trajectories(self):
        shp_c = (self.T, self.ncp, self.d)
        shp_v = (self.T, self.nv, self.d)
        out = [np.zeros(shp_c), np.zeros(shp_c), np.zeros(shp_v), np.zeros(shp_v), np.zeros(shp_c), np.zeros(shp_c)]
        self.ctx.check(self.ctx.lib.gbk_registration_trajectories(self.h, *[ctypes.c_void_p(a.ctypes.data) for a in out]))
        return dict(zip(("pos", "mom", "lm", "theta", "xi_pos", "xi_mom"), out))

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gbk_registration_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _objects_arrays(objects, d, kinds):
    """Per-object arrays of a multi-object description: kinds, point counts, concatenated points,
    cell counts, concatenated cells (int32, cell-free kinds contribute none)."""
    k = np.array([kinds[o["kind"]] for o in objects], dtype=np.int32)
    nv = np.array([len(o["pts"]) for o in objects], dtype=np.int64)
    pts = np.ascontiguousarray(np.concatenate([np.asarray(o["pts"], np.float64).reshape(-1, d) for o in objects]))
    cells, nc = [], []
    for o in objects:
        if o["kind"] in ("pointcloud", "landmark") or o.get("cells") is None:
            nc.append(len(o["pts"]))
        else:
            c = np.asarray(o["cells"], dtype=np.int32)
            nc.append(len(c))
            cells.append(c.reshape(-1))
    cells = np.ascontiguousarray(np.concatenate(cells) if cells else np.zeros(1, np.int32), dtype=np.int32)
    return k, nv, pts, np.array(nc, dtype=np.int64), cells


class MultiObjectAtlas:
    """DeterministicAtlas with a template of several objects (gbk_mo_atlas_*): `objects` is a list
    of dict(kind, pts, cells, sigma, sigma2) (kind as Registration.KINDS, sigma the data kernel width,
    sigma2 the data sigma^2), `subjects` a list over subjects of [(points, cells) per object]. One
    registration per subject, replayed from CUDA graphs; the optimiser deforms the reference's lagged
    template unless set_lagged_template(False)."""

    def __init__(self, ncp: int, objects, subjects, T: int, sigma_def: float, heun: bool = False,
                 context: Context | None = None):
        self.ctx = context or Context()
        self.d = int(np.asarray(objects[0]["pts"]).shape[1])
        self.ncp, self.S, self.nobj = int(ncp), len(subjects), len(objects)
        kinds, nv, pts, nc, cells = _objects_arrays(objects, self.d, Registration.KINDS)
        self.nv = int(nv.sum())
        sd = np.array([float(o["sigma"]) for o in objects])
        s2 = np.array([float(o["sigma2"]) for o in objects])
        tn, tp, tnc, tc = [], [], [], []
        for subj in subjects:
            if len(subj) != self.nobj:
                raise ValueError("every subject needs one target per template object")
            objs = [dict(o, pts=t[0], cells=t[1]) for o, t in zip(objects, subj)]
            _, n_t, p_t, c_n, c_t = _objects_arrays(objs, self.d, Registration.KINDS)
            tn.append(n_t), tp.append(p_t), tnc.append(c_n)
            if any(o["kind"] not in ("pointcloud", "landmark") for o in objects):
                tc.append(c_t)
        nv_t, ncell_t = np.concatenate(tn), np.concatenate(tnc)
        tgt = np.ascontiguousarray(np.concatenate(tp))
        tcells = np.ascontiguousarray(np.concatenate(tc) if tc else np.zeros(1, np.int32), dtype=np.int32)
        c = lambda a: ctypes.c_void_p(a.ctypes.data)
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.gbk_mo_atlas_create(
            self.ctx.h, self.d, self.ncp, self.nobj, c(kinds), c(nv), c(pts), c(nc), c(cells), c(sd), c(s2), self.S,
            c(nv_t), c(tgt), c(ncell_t), c(tcells), int(T), float(sigma_def), int(heun), ctypes.byref(h)))
        self.h = h

    def _check_shapes(self, cp, tmpl, mom):
        if cp.shape != (self.ncp, self.d) or tmpl.shape != (self.nv, self.d) or mom.shape != (self.S, self.ncp, self.d):
            raise ValueError(f"expected cp {(self.ncp, self.d)}, template {(self.nv, self.d)}, "
                             f"momenta {(self.S, self.ncp, self.d)}")

    def set_template_smoothing(self, width: float):
        self.ctx.check(self.ctx.lib.gbk_mo_atlas_set_template_smoothing(self.h, float(width)))

    def set_lagged_template(self, enable: bool):
        self.ctx.check(self.ctx.lib.gbk_mo_atlas_set_lagged_template(self.h, int(enable)))

    def step(self, cp, tmpl, mom):
        """Returns loglik [L, L_data, L_reg], dL/dcp, the smoothed template gradient, dL/dp."""
        cp, tmpl, mom = (np.ascontiguousarray(a, dtype=np.float64) for a in (cp, tmpl, mom))
        self._check_shapes(cp, tmpl, mom)
        ll = np.zeros(3)
        gc, gt, gm = np.zeros_like(cp), np.zeros_like(tmpl), np.zeros_like(mom)
        c = lambda a: ctypes.c_void_p(a.ctypes.data)
        self.ctx.check(self.ctx.lib.gbk_mo_atlas_step(self.h, c(cp), c(tmpl), c(mom), c(ll), c(gc), c(gt), c(gm)))
        return ll, gc, gt, gm

    def optimize(self, cp, tmpl, mom, max_iterations: int, initial_step: float = 1e-3, optimize_cp: bool = True,
                 optimize_template: bool = True, max_line_search: int = 10, shrink: float = 0.5, expand: float = 1.2,
                 tolerance: float = 1e-4, nb_iter_freeze: int = 3):
        """The context's estimator (FastGradientAscent by default, or GradientAscent) over [control
        points] [template] momenta on the device.
        Returns a dict like Atlas.optimize plus aux_* and grad_* (extrapolated point, gradient there)."""
        cp, tmpl, mom = (np.array(a, dtype=np.float64) for a in (cp, tmpl, mom))
        self._check_shapes(cp, tmpl, mom)
        hist = np.zeros((max_iterations + 1, 2))
        info = np.zeros(10)
        aux = [np.zeros_like(a) for a in (cp, tmpl, mom)]
        grd = [np.zeros_like(a) for a in (cp, tmpl, mom)]
        iters = ctypes.c_int(0)
        c = lambda a: ctypes.c_void_p(a.ctypes.data)
        self.ctx.check(self.ctx.lib.gbk_mo_atlas_optimize(
            self.h, c(cp), c(tmpl), c(mom), int(optimize_cp), int(optimize_template), int(max_iterations),
            float(initial_step), int(max_line_search), float(shrink), float(expand), float(tolerance),
            int(nb_iter_freeze), c(hist), ctypes.byref(iters), c(info), *[c(a) for a in aux], *[c(a) for a in grd]))
        groups = [k for k, on in (("cp", optimize_cp), ("template", optimize_template), ("momenta", True)) if on]
        idx = {"cp": (0, 5), "template": (1, 6), "momenta": (2, 7)}
        return {"cp": cp, "template": tmpl, "mom": mom, "aux_cp": aux[0], "aux_template": aux[1], "aux_mom": aux[2],
                "grad_cp": grd[0], "grad_template": grd[1], "grad_mom": grd[2], "history": hist[:iters.value],
                "step": np.array([info[idx[g][0]] for g in groups]), "tau": float(info[3]),
                "freeze_counter": int(info[4]), "grad_sq_norms": np.array([info[idx[g][1]] for g in groups]),
                "evaluations": int(info[8]), "stopped": Registration.STOP[int(info[9])]}

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gbk_mo_atlas_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GeodesicRegression:
    """The reference's geodesic Regression (gbk_geodesic_regression_*): `objects` as for
    MultiObjectAtlas, `observations` a list of [(points, cells) per object] at the time indices
    `times` of T time points over [t0, tn]. The gradient is the reference's unless
    set_corrected_gradient(True)."""

    def __init__(self, ncp: int, objects, observations, times, T: int, sigma_def: float, t0: float, tn: float,
                 heun: bool = False, context: Context | None = None):
        self.ctx = context or Context()
        self.d = int(np.asarray(objects[0]["pts"]).shape[1])
        self.ncp, self.nobs = int(ncp), len(observations)
        kinds, nv, pts, nc, cells = _objects_arrays(objects, self.d, Registration.KINDS)
        self.nv = int(nv.sum())
        sd = np.array([float(o["sigma"]) for o in objects])
        s2 = np.array([float(o["sigma2"]) for o in objects])
        tn_, tp, tnc, tc = [], [], [], []
        for ob in observations:
            objs = [dict(o, pts=t[0], cells=t[1]) for o, t in zip(objects, ob)]
            _, n_t, p_t, c_n, c_t = _objects_arrays(objs, self.d, Registration.KINDS)
            tn_.append(n_t), tp.append(p_t), tnc.append(c_n)
            if any(o["kind"] not in ("pointcloud", "landmark") for o in objects):
                tc.append(c_t)
        nv_t, ncell_t = np.concatenate(tn_), np.concatenate(tnc)
        tgt = np.ascontiguousarray(np.concatenate(tp))
        tcells = np.ascontiguousarray(np.concatenate(tc) if tc else np.zeros(1, np.int32), dtype=np.int32)
        ti = np.ascontiguousarray(times, dtype=np.int32)
        c = lambda a: ctypes.c_void_p(a.ctypes.data)
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.gbk_geodesic_regression_create(
            self.ctx.h, self.d, self.ncp, len(objects), c(kinds), c(nv), c(pts), c(nc), c(cells), c(sd), c(s2),
            self.nobs, c(ti), c(nv_t), c(tgt), c(ncell_t), c(tcells), int(T), float(sigma_def), float(t0), float(tn),
            int(heun), ctypes.byref(h)))
        self.h = h

    def set_template_smoothing(self, width: float):
        self.ctx.check(self.ctx.lib.gbk_geodesic_regression_set_template_smoothing(self.h, float(width)))

    def _check_shapes(self, cp, mom, tmpl):
        if cp.shape != (self.ncp, self.d) or mom.shape != (self.ncp, self.d) or (
                tmpl is not None and tmpl.shape != (self.nv, self.d)):
            raise ValueError(f"expected cp and momenta {(self.ncp, self.d)}, template {(self.nv, self.d)}")

    def set_corrected_gradient(self, enable: bool):
        self.ctx.check(self.ctx.lib.gbk_geodesic_regression_set_corrected_gradient(self.h, int(enable)))

    def step(self, cp, mom, tmpl=None):
        """Returns loglik [L, L_data, L_reg, sum of matches, <Kp,p>], dL/dcp, dL/dp, the smoothed
        template gradient."""
        cp, mom = np.ascontiguousarray(cp, np.float64), np.ascontiguousarray(mom, np.float64)
        t = None if tmpl is None else np.ascontiguousarray(tmpl, np.float64)
        self._check_shapes(cp, mom, t)
        ll = np.zeros(5)
        gc, gm, gt = np.zeros_like(cp), np.zeros_like(mom), np.zeros((self.nv, self.d))
        c = lambda a: None if a is None else ctypes.c_void_p(a.ctypes.data)
        self.ctx.check(self.ctx.lib.gbk_geodesic_regression_step(self.h, c(cp), c(mom), c(t), c(ll), c(gc), c(gm),
                                                                 c(gt)))
        return ll, gc, gm, gt

    def optimize(self, cp, mom, tmpl, max_iterations: int, initial_step: float = 1e-3, optimize_cp: bool = True,
                 optimize_template: bool = True, max_line_search: int = 10, shrink: float = 0.5, expand: float = 1.2,
                 tolerance: float = 1e-4, nb_iter_freeze: int = 3):
        cp, mom, tmpl = (np.array(a, dtype=np.float64) for a in (cp, mom, tmpl))
        self._check_shapes(cp, mom, tmpl)
        hist = np.zeros((max_iterations + 1, 2))
        info = np.zeros(10)
        aux = [np.zeros_like(a) for a in (cp, mom, tmpl)]
        grd = [np.zeros_like(a) for a in (cp, mom, tmpl)]
        iters = ctypes.c_int(0)
        c = lambda a: ctypes.c_void_p(a.ctypes.data)
        self.ctx.check(self.ctx.lib.gbk_geodesic_regression_optimize(
            self.h, c(cp), c(mom), c(tmpl), int(optimize_cp), int(optimize_template), int(max_iterations),
            float(initial_step), int(max_line_search), float(shrink), float(expand), float(tolerance),
            int(nb_iter_freeze), c(hist), ctypes.byref(iters), c(info), *[c(a) for a in aux], *[c(a) for a in grd]))
        groups = [k for k, on in (("cp", optimize_cp), ("momenta", True), ("template", optimize_template)) if on]
        idx = {"cp": (0, 5), "momenta": (1, 6), "template": (2, 7)}
        return {"cp": cp, "mom": mom, "template": tmpl, "aux_cp": aux[0], "aux_mom": aux[1], "aux_template": aux[2],
                "grad_cp": grd[0], "grad_mom": grd[1], "grad_template": grd[2], "history": hist[:iters.value],
                "step": np.array([info[idx[g][0]] for g in groups]), "tau": float(info[3]),
                "freeze_counter": int(info[4]), "grad_sq_norms": np.array([info[idx[g][1]] for g in groups]),
                "evaluations": int(info[8]), "stopped": Registration.STOP[int(info[9])]}

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gbk_geodesic_regression_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Atlas:
    """DeterministicAtlas iteration over many subjects, every stage one launch for all subjects
    (uneven target meshes balanced by source chunks), replayed from a CUDA graph."""

    KINDS = {"currents": 0, "varifold": 1}

    def __init__(self, cp, tmpl_pts, tmpl_tris, targets, T: int, sigma_def: float, sigma_data: float,
                 data_sigma2: float, kind: str = "currents", heun: bool = True, context: Context | None = None):
        self.ctx = context or Context()
        cp = np.ascontiguousarray(cp, dtype=np.float64)
        tp, tt = np.ascontiguousarray(tmpl_pts, np.float64), np.ascontiguousarray(tmpl_tris, np.int32)
        self.S, self.ncp, self.nv = len(targets), cp.shape[0], tp.shape[0]
        nv_t = np.array([t[0].shape[0] for t in targets], dtype=np.int64)
        nf_t = np.array([t[1].shape[0] for t in targets], dtype=np.int64)
        pts = np.ascontiguousarray(np.concatenate([t[0] for t in targets]), np.float64)
        tris = np.ascontiguousarray(np.concatenate([t[1] for t in targets]), np.int32)
        h = ctypes.c_void_p()
        c = lambda a: ctypes.c_void_p(a.ctypes.data)
        self.ctx.check(self.ctx.lib.gbk_atlas_create(
            self.ctx.h, self.ncp, c(cp), self.nv, c(tp), tt.shape[0], c(tt), self.S, c(nv_t), c(pts), c(nf_t),
            c(tris), int(T), float(sigma_def), float(sigma_data), float(data_sigma2), self.KINDS[kind], int(heun),
            ctypes.byref(h)))
        self.h = h

    def set_lagged_template(self, enable: bool):
        """True (default): optimize() deforms the reference's lagged template (gbk_atlas_set_lagged_template)."""
        self.ctx.check(self.ctx.lib.gbk_atlas_set_lagged_template(self.h, int(enable)))

    def set_graph(self, enable: bool):
        self.ctx.check(self.ctx.lib.gbk_atlas_set_graph(self.h, int(enable)))

    def step(self, mom):
        """mom: S x ncp x 3. Returns loglik (3 + S), dL/dp (S x ncp x 3), dL/dcp, template gradient."""
        mom = np.ascontiguousarray(mom, dtype=np.float64)
        if mom.shape != (self.S, self.ncp, 3):
            raise ValueError(f"expected momenta of shape {(self.S, self.ncp, 3)}")
        ll = np.zeros(3 + self.S)
        gm = np.zeros((self.S, self.ncp, 3))
        gc = np.zeros((self.ncp, 3))
        gt = np.zeros((self.nv, 3))
        c = lambda a: ctypes.c_void_p(a.ctypes.data)
        self.ctx.check(self.ctx.lib.gbk_atlas_step(self.h, c(mom), c(ll), c(gm), c(gc), c(gt)))
        return ll, gm, gc, gt

    def graph_launches(self) -> int:
        return int(self.ctx.lib.gbk_atlas_graph_launches(self.h))

    def set_template_smoothing(self, width: float):
        """Template-gradient smoothing width (ConvolveGradTemplate); 0 = the L2 gradient."""
        self.ctx.check(self.ctx.lib.gbk_atlas_set_template_smoothing(self.h, float(width)))

    def optimize(self, cp, tmpl, mom, max_iterations: int, initial_step: float = 1e-3, optimize_cp: bool = True,
                 optimize_template: bool = True, max_line_search: int = 10, shrink: float = 0.5,
                 expand: float = 1.2, tolerance: float = 1e-4, nb_iter_freeze: int = 3):
        """The context's estimator (the reference's FastGradientAscent by default, or its
        GradientAscent: Context.set_estimator) over control points, template points and momenta, on
        the device (gbk_atlas_optimize). Returns a dict: cp, tmpl, mom (final), history, step and
        grad_sq_norms per optimised group, tau, freeze_counter, evaluations, stopped."""
        cp, tmpl, mom = (np.array(v, dtype=np.float64) for v in (cp, tmpl, mom))
        if cp.shape != (self.ncp, 3) or tmpl.shape != (self.nv, 3) or mom.shape != (self.S, self.ncp, 3):
            raise ValueError(f"expected cp {(self.ncp, 3)}, template {(self.nv, 3)}, momenta {(self.S, self.ncp, 3)}")
        hist = np.zeros((max_iterations + 1, 2))
        info = np.zeros(10)
        iters = ctypes.c_int(0)
        c = lambda a: ctypes.c_void_p(a.ctypes.data)
        self.ctx.check(self.ctx.lib.gbk_atlas_optimize(
            self.h, c(cp), c(tmpl), c(mom), int(optimize_cp), int(optimize_template), int(max_iterations),
            float(initial_step), int(max_line_search), float(shrink), float(expand), float(tolerance),
            int(nb_iter_freeze), c(hist), ctypes.byref(iters), c(info)))
        groups = [g for g, on in ((0, optimize_cp), (1, optimize_template), (2, True)) if on]
        return {"cp": cp, "tmpl": tmpl, "mom": mom, "history": hist[:iters.value], "step": info[groups],
                "grad_sq_norms": info[[5 + g for g in groups]], "tau": float(info[3]),
                "freeze_counter": int(info[4]), "evaluations": int(info[8]),
                "stopped": Registration.STOP[int(info[9])]}

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gbk_atlas_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
