"""Restatement of the reference's FastGradientAscent estimator (test infrastructure only: the
oracle for the library's device-resident registration optimiser).

Follows src/core/estimators/FastGradientAscent.cxx:48-300 (Update: Nesterov-accelerated gradient
ascent with a per-parameter-group step size, multivariate line search, step expansion after
m_NbIterFreeze accepted first trials, stop on the relative log-likelihood change) and :306-335
(GradientAscentStep). Defaults are the reference's: FastGradientAscent.cxx:22 (NbIterFreeze 3,
multivariate line search on) and SparseDiffeoParameters.cxx:75-82 (10 line-search iterations,
expand 1.2, shrink 0.5, tolerance 1e-4).

`evaluate(params, need_grad)` returns (terms, grads, grad_sq_norms): terms = [data, regularity]
log-likelihood terms at `params` (a list of arrays, one per parameter group, in the reference's
order: population effects alphabetically, then individual ones), and, when need_grad, the
gradient of each group and the squared norm the reference weights the step with
(DeterministicAtlas.cxx:230-234).
"""
from __future__ import annotations

import math

import numpy as np


def fast_gradient_ascent(evaluate, params, initial_step: float, max_iterations: int,
                         max_line_search: int = 10, shrink: float = 0.5, expand: float = 1.2,
                         tolerance: float = 1e-4, nb_iter_freeze: int = 3, multivariate: bool = True,
                         set_fixed=None):
    """set_fixed(params), when given, is called wherever the reference calls
    SetFixedEffects (before every evaluation at a new point, and around the per-iteration state
    write, SaveEveryNIters = 1 by default, SparseDiffeoParameters.cxx:105), for models whose state
    depends on that sequence; the log-likelihood at the extrapolated point and the gradient there
    are then two evaluations, as in the reference (:245-258)."""
    fixed = [np.array(p, dtype=np.float64) for p in params]
    aux = [p.copy() for p in fixed]
    history = [None] * (max_iterations + 1)
    sf = set_fixed or (lambda p: None)
    if set_fixed is None:
        terms0, grads, sq = evaluate(aux, True)
    else:
        terms0 = evaluate(aux, False)[0]
        _, grads, sq = evaluate(aux, True)
    history[0] = np.asarray(terms0, dtype=np.float64)
    lsq_ref = float(np.sum(history[0]))
    n = len(fixed)
    step = np.full(n, float(initial_step))
    tau = 1.0
    freeze = 1
    evaluations = 1
    it = 1
    stopped = "max_iterations"

    def ascent(local_step):  # GradientAscentStep, :306-335
        return [aux[k] + grads[k] * local_step[k] for k in range(n)]

    while it < max_iterations + 1:
        found = False
        new = None
        new_terms = None
        for li in range(max_line_search):
            cand = ascent(step)
            sf(cand)
            t, _, _ = evaluate(cand, False)
            evaluations += 1
            q = float(np.sum(t)) - lsq_ref - float(np.dot(sq, step)) * shrink
            if q >= 0:
                found, new, new_terms = True, cand, np.asarray(t, dtype=np.float64)
                if li == 0:
                    freeze += 1
                break
            elif n > 1 and multivariate:
                freeze = 1
                step = step * shrink
                props, qs, ts = [], np.empty(n), []
                for k in range(n):
                    local = step.copy()
                    local[k] /= shrink
                    ck = ascent(local)
                    sf(ck)
                    tk, _, _ = evaluate(ck, False)
                    evaluations += 1
                    props.append(ck)
                    ts.append(np.asarray(tk, dtype=np.float64))
                    qs[k] = float(np.sum(tk)) - lsq_ref - float(np.dot(sq, local)) * shrink
                idx = int(np.argmax(qs))
                if qs[idx] >= 0:
                    new, new_terms = props[idx], ts[idx]
                    step[idx] /= shrink
                    found = True
                    break
            else:
                freeze = 1
                step = step * shrink
        if not found:
            sf(fixed)
            stopped = "line_search"
            break
        history[it] = new_terms
        tau_next = (1.0 + math.sqrt(1.0 + 4.0 * tau * tau)) / 2.0
        if freeze > nb_iter_freeze:
            step = step * expand
            tau_next = (1.0 + math.sqrt(1.0 + 4.0 * tau * tau / expand)) / 2.0
        tau_scale = (tau - 1.0) / tau_next
        aux = [new[k] + (new[k] - fixed[k]) * tau_scale for k in range(n)]
        fixed = new
        tau = tau_next
        if set_fixed is None:
            t_aux, grads, sq = evaluate(aux, True)
        else:
            sf(aux)
            t_aux = evaluate(aux, False)[0]
            sf(fixed)  # the state write of every iteration (:250-254)
            sf(aux)
            _, grads, sq = evaluate(aux, True)
        evaluations += 1
        lsq_ref = float(np.sum(t_aux))
        d_cur = float(np.sum(history[it - 1]) - np.sum(history[it]))
        d_ref = float(np.sum(history[0]) - np.sum(history[it]))
        if abs(d_cur) < tolerance * abs(d_ref):
            stopped = "tolerance"
            it += 1
            break
        it += 1
    sf(fixed)
    done = [h for h in history if h is not None]
    return {"params": fixed, "aux": aux, "grads": grads, "grad_sq_norms": np.asarray(sq, dtype=np.float64),
            "step": step, "tau": tau, "freeze_counter": freeze, "iter": it, "history": np.stack(done),
            "evaluations": evaluations, "stopped": stopped}


def gradient_ascent(evaluate, params, initial_step: float, max_iterations: int, max_line_search: int = 10,
                    shrink: float = 0.5, expand: float = 1.2, tolerance: float = 1e-4, multivariate: bool = True,
                    set_fixed=None):
    """The reference's GradientAscent estimator (GradientAscent.cxx:48-240): from the fixed point,
    a trial fixed + grad * step is accepted when its log-likelihood is not below the current one
    (no sufficient-increase term); otherwise every step shrinks and, with several groups, the
    "all but one shrunk" proposals are tried and the best acceptable one kept (its group's step
    restored); after an accepted step every step expands; stop on |dL| < tolerance |L_0 - L| or when
    the line search fails. The gradient is evaluated at each new fixed point. set_fixed as in
    fast_gradient_ascent (the reference calls SetFixedEffects before every trial and before each
    gradient, :154-218)."""
    fixed = [np.array(p, dtype=np.float64) for p in params]
    sf = set_fixed or (lambda p: None)
    history = [None] * (max_iterations + 1)
    t0, _, _ = evaluate(fixed, False)
    history[0] = np.asarray(t0, dtype=np.float64)
    lsq_ref = float(np.sum(history[0]))
    _, grads, sq = evaluate(fixed, True)
    n = len(fixed)
    step = np.full(n, float(initial_step))
    evaluations, it, stopped = 2, 1, "max_iterations"
    step_at = lambda local: [fixed[k] + grads[k] * local[k] for k in range(n)]
    while it < max_iterations + 1:
        found = False
        for li in range(max_line_search):
            cand = step_at(step)
            sf(cand)
            t, _, _ = evaluate(cand, False)
            evaluations += 1
            if float(np.sum(t)) - lsq_ref >= 0:
                found, new, new_terms = True, cand, np.asarray(t, dtype=np.float64)
                break
            elif n > 1 and multivariate:
                step = step * shrink
                props, ts, qs = [], [], np.empty(n)
                for k in range(n):
                    local = step.copy()
                    local[k] /= shrink
                    ck = step_at(local)
                    sf(ck)
                    tk, _, _ = evaluate(ck, False)
                    evaluations += 1
                    props.append(ck)
                    ts.append(np.asarray(tk, dtype=np.float64))
                    qs[k] = float(np.sum(tk)) - lsq_ref
                idx = int(np.argmax(qs))
                if qs[idx] >= 0:
                    found, new, new_terms = True, props[idx], ts[idx]
                    step[idx] /= shrink
                    break
            else:
                step = step * shrink
        if not found:
            sf(fixed)
            stopped = "line_search"
            break
        history[it] = new_terms
        fixed = new
        step = step * expand
        lsq_ref = float(np.sum(new_terms))
        d_cur = float(np.sum(history[it - 1]) - np.sum(history[it]))
        d_ref = float(np.sum(history[0]) - np.sum(history[it]))
        if abs(d_cur) < tolerance * abs(d_ref):
            stopped = "tolerance"
            break
        sf(fixed)
        _, grads, sq = evaluate(fixed, True)
        evaluations += 1
        it += 1
    done = [h for h in history if h is not None]
    return {"params": fixed, "grads": grads, "grad_sq_norms": np.asarray(sq, dtype=np.float64), "step": step,
            "iter": it, "history": np.stack(done), "evaluations": evaluations, "stopped": stopped}


def registration_evaluator(K, tmpl_pts, tmpl_tris, tgt_pts, tgt_tris, T: int, sigma_def: float,
                           sigma_data: float, data_sigma2: float, kind: str = "currents", heun: bool = True):
    """evaluate() of one landmark registration with control points and momenta optimised (the
    reference's DeterministicAtlas with one subject and a frozen template): parameter groups
    [ControlPoints, Momenta]."""
    from .deformation import registration

    def evaluate(params, need_grad):
        cp, mom = params
        L, g_cp, g_mom, info = registration(K, cp, mom, tmpl_pts, tmpl_tris, tgt_pts, tgt_tris, T, sigma_def,
                                            sigma_data, data_sigma2, kind=kind, heun=heun)
        data = -0.5 * info["match"] / data_sigma2
        terms = [data, L - data]
        if not need_grad:
            return terms, None, None
        return terms, [g_cp, g_mom], np.array([float(np.sum(g_cp * g_cp)), float(np.sum(g_mom * g_mom))])

    return evaluate


def atlas_evaluator(K, tmpl_cells, targets, T: int, sigma_def: float, sigma_data: float, data_sigma2: float,
                    kind: str = "currents", heun: bool = True, smoothing_width: float = 0.0,
                    optimize_cp: bool = True, optimize_template: bool = True, cp=None, tmpl=None, lag=None):
    """evaluate() of a DeterministicAtlas over the subjects `targets` ([(points, cells)]): parameter
    groups in the reference's order [ControlPoints] [TemplateData] Momenta (one ncp x d block per
    subject, stacked). The template gradient is the sum over subjects of -theta_s(0)
    (AbstractAtlas.cxx:559-613) smoothed by a Gaussian of width smoothing_width over the template
    points (ConvolveGradTemplate, :724-748; no smoothing at width 0), and its squared norm is
    <L2, smoothed> (DeterministicAtlas.cxx:232). Frozen groups take their values from `cp` /
    `tmpl`. With `lag` (a LaggedTemplate) the subjects deform the reference's lagged template."""
    from .deformation import registration
    cp_frozen, tmpl_frozen = cp, tmpl

    def evaluate(params, need_grad):
        k = 0
        cp = params[k] if optimize_cp else cp_frozen
        k += int(optimize_cp)
        tmpl = params[k] if optimize_template else tmpl_frozen
        k += int(optimize_template)
        mom = params[k]
        data = reg = 0.0
        g_cp = np.zeros_like(cp)
        g_t = np.zeros_like(tmpl)
        g_mom = np.zeros_like(mom)
        moved = tmpl if lag is None or not optimize_template else lag.deformed
        for s, (pts, cells) in enumerate(targets):
            L, gc, gm, info = registration(K, cp, mom[s], moved, tmpl_cells, pts, cells, T, sigma_def, sigma_data,
                                           data_sigma2, kind=kind, heun=heun)
            d_s = -0.5 * info["match"] / data_sigma2
            data += d_s
            reg += L - d_s
            g_cp += gc
            g_mom[s] = gm
            g_t -= info["theta"][0]
        terms = [data, reg]
        if not need_grad:
            return terms, None, None
        grads, sq = [], []
        if optimize_cp:
            grads.append(g_cp)
            sq.append(float(np.sum(g_cp * g_cp)))
        if optimize_template:
            sob = K.convolve(tmpl, tmpl, g_t, smoothing_width) if smoothing_width >= 1e-20 else g_t
            grads.append(sob)
            sq.append(float(np.sum(g_t * sob)))
        grads.append(g_mom)
        sq.append(float(np.sum(g_mom * g_mom)))
        return terms, grads, np.array(sq)

    return evaluate


class LaggedTemplate:
    """The template the reference deforms during an atlas estimation. AbstractAtlas::SetFixedEffects
    (AbstractAtlas.cxx:52-65) reads the template data of the fixed effects BEFORE storing the new
    map and writes that older copy into the template objects, so every evaluation deforms the
    template of the previous SetFixedEffects call, while the smoothing of the template gradient
    (ConvolveGradTemplate, :724-748) and the step use the current one. set_fixed(params) follows
    the calls; `deformed` is the template the next evaluation deforms."""

    def __init__(self, tmpl, index: int):
        self.current = np.array(tmpl, dtype=np.float64)
        self.deformed = self.current.copy()
        self.index = index

    def set_fixed(self, params):
        self.deformed = self.current
        self.current = np.array(params[self.index], dtype=np.float64)


def multi_object_atlas_evaluator(K, objects, subjects, T: int, sigma_def: float, heun: bool = False,
                                 smoothing_width: float = 0.0, optimize_cp: bool = True,
                                 optimize_template: bool = True, cp=None, tmpl=None, lag: LaggedTemplate = None):
    """evaluate() of a DeterministicAtlas with a multi-object template: objects[i] = dict(kind,
    cells, sigma, sigma2, n) in template order (the template points are the objects' points
    concatenated), subjects[s][i] = (points, cells) of object i of subject s. Groups as in
    atlas_evaluator. Per subject the data term sums its objects (DeterministicAtlas.cxx:121-125:
    subjects outer, objects inner, then * 0.5); the template gradient is sum_s -theta_s(0), smoothed
    object by object on that object's own points (ConvolveGradTemplate, AbstractAtlas.cxx:724-748),
    and its squared norm is the sum over objects of <L2, smoothed> (DeterministicAtlas.cxx:232).
    With `lag` (a LaggedTemplate whose set_fixed goes to fast_gradient_ascent) the deformation uses
    the lagged template as the reference does."""
    from .deformation import registration_multi
    cp_frozen, tmpl_frozen = cp, tmpl
    offs = np.cumsum([0] + [ob["n"] for ob in objects])

    def evaluate(params, need_grad):
        k = 0
        cp = params[k] if optimize_cp else cp_frozen
        k += int(optimize_cp)
        tmpl = params[k] if optimize_template else tmpl_frozen
        k += int(optimize_template)
        mom = params[k]
        data = reg = 0.0
        g_cp = np.zeros_like(cp)
        g_t = np.zeros_like(tmpl)
        g_mom = np.zeros_like(mom)
        moved = tmpl if lag is None or not optimize_template else lag.deformed
        for s, targets in enumerate(subjects):
            d_s, r_s, gc, gm, info = registration_multi(K, cp, mom[s], moved, objects, targets, T, sigma_def, heun)
            data += d_s
            reg += r_s
            g_cp += gc
            g_mom[s] = gm
            g_t -= info["theta"][0]
        terms = [data, reg]
        if not need_grad:
            return terms, None, None
        grads, sq = [], []
        if optimize_cp:
            grads.append(g_cp)
            sq.append(float(np.sum(g_cp * g_cp)))
        if optimize_template:
            sob = g_t.copy()
            if smoothing_width >= 1e-20:
                for i in range(len(objects)):
                    a, b = offs[i], offs[i + 1]
                    sob[a:b] = K.convolve(tmpl[a:b], tmpl[a:b], g_t[a:b], smoothing_width)
            grads.append(sob)
            sq.append(float(sum(np.sum(g_t[offs[i]:offs[i + 1]] * sob[offs[i]:offs[i + 1]])
                                for i in range(len(objects)))))
        grads.append(g_mom)
        sq.append(float(np.sum(g_mom * g_mom)))
        return terms, grads, np.array(sq)

    return evaluate


def regression_evaluator(K, objects, observations, times, T: int, sigma_def: float, t0: float, tn: float,
                         heun: bool = False, smoothing_width: float = 0.0, corrected: bool = False):
    """evaluate() of the reference's geodesic Regression (oracle.deformation.geodesic_regression) for
    fast_gradient_ascent: groups in the reference's order ControlPoints, InitialMomenta, TemplateData
    (Regression.cxx:279-286); the template gradient smoothed object by object
    (Regression::ConvolveGradTemplate, :688-712); squared norms |g_cp|^2, |g_mom|^2, <L2, smoothed>.
    Regression::SetFixedEffects (:55-66) writes the new template into the template objects, so no
    lag."""
    from .deformation import geodesic_regression
    offs = np.cumsum([0] + [ob["n"] for ob in objects])

    def evaluate(params, need_grad):
        cp, mom, tmpl = params
        data, reg, g_cp, g_mom, g_t, _ = geodesic_regression(K, cp, mom, tmpl, objects, observations, times, T,
                                                             sigma_def, t0, tn, heun, corrected)
        if not need_grad:
            return [data, reg], None, None
        sob = g_t.copy()
        if smoothing_width >= 1e-20:
            for i in range(len(objects)):
                a, b = offs[i], offs[i + 1]
                sob[a:b] = K.convolve(tmpl[a:b], tmpl[a:b], g_t[a:b], smoothing_width)
        sq = np.array([float(np.sum(g_cp * g_cp)), float(np.sum(g_mom * g_mom)), float(np.sum(g_t * sob))])
        return [data, reg], [g_cp, g_mom, sob], sq

    return evaluate


def initial_control_points(points, spacing: float):
    """Regular grid over a bounding box (AbstractAtlas.cxx:240-330 without the image criterion):
    per axis, spacing apart, centred so the leftover extent is split evenly; x outermost."""
    lo, hi = np.min(points, axis=0), np.max(points, axis=0)
    axes = []
    for d in range(points.shape[1]):
        off = 0.5 * (hi[d] - lo[d] - spacing * math.floor((hi[d] - lo[d]) / spacing))
        v, x = [], lo[d] + off
        while x <= hi[d]:
            v.append(x)
            x += spacing
        axes.append(v)
    mesh = np.meshgrid(*axes, indexing="ij")
    return np.stack([m.ravel() for m in mesh], axis=1)
