"""FP64 restatement of the reference's deformation loops (TEST INFRASTRUCTURE ONLY).

Diffeos, AdjointEquationsIntegrator and the atlas model need VTK/ITK/Boost and cannot be built
here, so their loops are restated in numpy, calling the kernel oracle (gauss_oracle.c, pinned to
the reference's compiled ExactKernel) for every kernel sum, exactly as the reference calls its
kernel object. Each function cites the reference lines it follows. The shooting loop is pinned by
the reference's parallel-transport golden test (tests/unit_tests/parallel-transport), which this
module also restates.
"""
from __future__ import annotations

import numpy as np

from .kernels import OracleLib


def _dt(T: int, t0: float = 0.0, tn: float = 1.0) -> float:
    return (tn - t0) / (T - 1)


def shoot(K: OracleLib, sigma: float, cp0, mom0, T: int, t0=0.0, tn=1.0):
    """Diffeos::Shoot, Diffeos.cxx:589-660: explicit Euler on the Hamiltonian system.
    x' = K(x,x) p ; p' = -dMom with dMom_i = G_i^T p_i (G = ConvolveGradient(X) varlin)."""
    cp0, mom0 = np.asarray(cp0, float), np.asarray(mom0, float)
    pos = [cp0.copy() for _ in range(T)]
    mom = [np.zeros_like(mom0) for _ in range(T)]
    mom[0] = mom0.copy()
    if np.linalg.norm(mom0) < 1e-20:  # :611-613
        return pos, mom
    dt = _dt(T, t0, tn)
    for t in range(T - 1):
        G = K.grad_varlin(pos[t], pos[t], mom[t], sigma)          # :624
        dpos = K.convolve(pos[t], pos[t], mom[t], sigma)          # :626
        dmom = np.einsum("ikl,ik->il", G, mom[t])                 # :627-630
        pos[t + 1] = pos[t] + dpos * dt                           # :631
        mom[t + 1] = mom[t] - dmom * dt                           # :632
    return pos, mom


def flow_landmarks(K: OracleLib, sigma: float, pos, mom, lm0, heun: bool = True, t0=0.0, tn=1.0):
    """Diffeos::FlowLandmarkPointsTrajectory, Diffeos.cxx:661-712 (Heun when ImprovedEuler)."""
    T = len(pos)
    lm = [np.asarray(lm0, float).copy() for _ in range(T)]
    if np.linalg.norm(mom[0]) < 1e-20:  # :683-684
        return lm
    dt = _dt(T, t0, tn)
    for t in range(T - 1):
        v = K.convolve(lm[t], pos[t], mom[t], sigma)              # :690
        lm[t + 1] = lm[t] + v * dt                                # :691
        if heun:
            v2 = K.convolve(lm[t + 1], pos[t + 1], mom[t + 1], sigma)  # :697
            lm[t + 1] = lm[t] + (v + v2) * (dt * 0.5)             # :698-699
    return lm


def adjoint_landmarks(K: OracleLib, sigma: float, pos, mom, lm, theta_final, heun: bool = True,
                      t0=0.0, tn=1.0):
    """AdjointEquationsIntegrator::IntegrateAdjointOfLandmarkPointsEquations, :59-136 (no jumps)."""
    T = len(pos)
    dt = _dt(T, t0, tn)
    theta = [None] * T
    theta[T - 1] = np.asarray(theta_final, float).copy()          # :91
    for t in range(T - 1, 0, -1):
        dth = K.grad_alpha(lm[t], pos[t], mom[t], sigma, theta[t])          # :106
        theta[t - 1] = theta[t] + dth * dt                                  # :117
        if heun:
            dth2 = K.grad_alpha(lm[t - 1], pos[t - 1], mom[t - 1], sigma, theta[t - 1])  # :126
            theta[t - 1] = theta[t] + (dth + dth2) * (dt * 0.5)             # :137
    return theta


def compute_update_at(K: OracleLib, sigma: float, pos_s, mom_s, xipos_s, ximom_s, lm_s=None,
                      theta_s=None):
    """AdjointEquationsIntegrator::ComputeUpdateAt, :476-570, landmark points only.
    Returns (dPos, dMom) = (dXi1 + dXi3 + dXi4, dXi2 + dXi5 + dXi6), with the seven kernel calls
    of the reference."""
    d = pos_s.shape[1]
    if lm_s is not None and lm_s.shape[0] > 0:
        dxi1 = K.grad_alpha(pos_s, lm_s, theta_s, sigma, mom_s)              # :519
        dxi2 = K.convolve(pos_s, lm_s, theta_s, sigma)                       # :521
    else:
        dxi1 = np.zeros_like(pos_s)
        dxi2 = np.zeros_like(pos_s)
    axipos = np.concatenate([mom_s, xipos_s], axis=1)                       # :523-525
    kaxipos = K.convolve(pos_s, pos_s, axipos, sigma)                        # :530
    gradax = K.grad_varlin(pos_s, pos_s, axipos, sigma)                      # :532 (n, 2d, d)
    gmom, gxip = gradax[:, :d, :], gradax[:, d:, :]
    dxi3 = np.einsum("ikl,ik->il", gmom, xipos_s) + np.einsum("ikl,ik->il", gxip, mom_s)  # :534-540
    dxi5 = kaxipos[:, d:]                                                    # :542
    dxi6 = np.zeros_like(pos_s)
    for dim in range(d):                                                     # :546-556
        W = ximom_s[:, dim:dim + 1] * mom_s
        dxi6 += K.grad_dim(pos_s, pos_s, W, sigma, dim)
    dxi6 -= np.einsum("ikl,il->ik", gmom, ximom_s)                           # :558-562
    dxi4 = K.special_hessian(pos_s, mom_s, sigma, ximom_s)                   # :564-566
    return dxi1 + dxi3 + dxi4, dxi2 + dxi5 + dxi6                            # :570-571


def adjoint_diffeo(K: OracleLib, sigma: float, pos, mom, lm=None, theta=None, heun: bool = True,
                   t0=0.0, tn=1.0):
    """AdjointEquationsIntegrator::IntegrateAdjointOfDiffeoParametersEquations, :414-470."""
    T = len(pos)
    dt = _dt(T, t0, tn)
    xp = [np.zeros_like(pos[0]) for _ in range(T)]                           # :421-425
    xm = [np.zeros_like(pos[0]) for _ in range(T)]
    L = (lambda s: lm[s]) if lm is not None else (lambda s: None)
    TH = (lambda s: theta[s]) if theta is not None else (lambda s: None)
    for t in range(T - 1, 0, -1):
        dp, dm = compute_update_at(K, sigma, pos[t], mom[t], xp[t], xm[t], L(t), TH(t))
        xp[t - 1] = xp[t] + dp * dt
        xm[t - 1] = xm[t] + dm * dt
        if heun:
            dp2, dm2 = compute_update_at(K, sigma, pos[t - 1], mom[t - 1], xp[t - 1], xm[t - 1],
                                         L(t - 1), TH(t - 1))
            xp[t - 1] = xp[t] + (dp + dp2) * (dt * 0.5)
            xm[t - 1] = xm[t] + (dm + dm2) * (dt * 0.5)
    return xp, xm


def parallel_transport(K: OracleLib, sigma: float, pos, mom, initial_momenta, initial_cp,
                       initial_time, target_times, t0=0.0, tn=1.0):
    """Diffeos::ParallelTransport, Diffeos.cxx:293-585 (ConvolveInverse by a dense FP64 solve,
    ExactKernel.cxx:154-164)."""
    T = len(pos)
    h = (tn - t0) / (T - 1)
    eps = h
    if (np.sum(mom[0] ** 2) < 1e-20 or np.sum(initial_momenta ** 2) < 1e-20 or not target_times
            or T <= 1):
        return [initial_momenta.copy() for _ in target_times]

    def to_index(tm):
        c = (tm - t0) / h
        i = int(c)
        return i + 1 if (c - i) >= 0.5 else i

    i0 = to_index(initial_time)
    tidx = [to_index(tm) for tm in target_times]
    fin = tidx[-1]
    nsteps = fin - i0 + 1
    if fin == i0:
        return [initial_momenta.copy() for _ in target_times]

    def conv_inverse(src, rhs):
        D = src[:, None, :] - src[None, :, :]
        Kmat = np.exp(-np.sum(D * D, axis=2) / sigma ** 2)
        return np.linalg.solve(Kmat, rhs)

    v0 = K.convolve(pos[0], initial_cp, initial_momenta, sigma)
    vel = [v0.copy() for _ in range(nsteps)]
    pt = [None] * nsteps
    ispwv = isnw = spwv = snw = snv = 0.0
    alpha, beta = 1.0, 0.0
    dot = lambda a, b: float(np.sum(a * b))
    idx = 0
    for t in range(i0, fin):
        dpos = K.convolve(pos[t], pos[t], mom[t], sigma)
        kinv = conv_inverse(pos[t], vel[idx])
        if t == i0:
            ispwv = dot(kinv, K.convolve(pos[t], pos[t], mom[t], sigma))
            isnw = dot(kinv, K.convolve(pos[t], pos[t], kinv, sigma))
        if t > i0:
            kk = K.convolve(pos[t], pos[t], kinv, sigma)
            pns = dot(kinv, kk)
            pspv = dot(mom[t], kk)
            alpha = np.sqrt((isnw * snv - ispwv * spwv) / (pns * snv - pspv * pspv))
            beta = (ispwv - alpha * pspv) / snv
        pt[idx] = alpha * kinv + beta * mom[t]
        kk = K.convolve(pos[t], pos[t], pt[idx], sigma)
        spwv = dot(mom[t], kk)
        snw = dot(kinv, kk)
        snv = dot(mom[t], K.convolve(pos[t], pos[t], mom[t], sigma))
        mp = mom[t] + eps * kinv
        mn = mom[t] - eps * kinv
        Gp = K.grad_varlin(pos[t], pos[t], mp, sigma)
        dmp = np.einsum("ikl,ik->il", Gp, mp)
        Gn = K.grad_varlin(pos[t], pos[t], mn, sigma)
        dmn = np.einsum("ikl,ik->il", Gn, mn)
        div = 1.0 / (2 * eps)
        c1 = pos[t] + h / 2 * (dpos + eps * vel[idx])
        m1 = mp - h / 2 * dmp
        cplus = (pos[t] + h * K.convolve(c1, c1, m1, sigma)) * div
        c1 = pos[t] + h / 2 * (dpos - eps * vel[idx])
        m1 = mn - h / 2 * dmn
        cminus = (pos[t] + h * K.convolve(c1, c1, m1, sigma)) * div
        vel[idx + 1] = (cplus - cminus) / eps
        idx += 1
    pt[idx] = conv_inverse(pos[fin - 1], vel[idx])   # quirk kept: kernel at finalIndex - 1
    out, oi = [], 0
    for t in range(i0, fin + 1):
        if oi < len(tidx) and t == tidx[oi]:
            out.append(pt[t - i0])
            oi += 1
    return out


def registration(K: OracleLib, cp, mom, tmpl_pts, tmpl_tris, tgt_pts, tgt_tris, T: int,
                 sigma_def: float, sigma_data: float, data_sigma2: float, kind: str = "currents",
                 heun: bool = True):
    """Log-likelihood and gradient of one subject of DeterministicAtlas with a frozen template.

    L = -0.5 match / data_sigma2 - 0.5 <K p, p>   (DeterministicAtlas.cxx:99-154)
    dL/dp = -xi_mom(0) - K p ; dL/dcp = -xi_pos(0) - ConvolveGradient(cp, p)
    (AbstractAtlas.cxx:559-613 with the adjoint seeded by the match gradient / (2 data_sigma2);
    DeterministicAtlas::AddGradientRegularityTerm, :246-280).
    """
    from . import geometry as G
    match_f, grad_f = G.KINDS[kind]
    pos, mo = shoot(K, sigma_def, cp, mom, T)
    lm = flow_landmarks(K, sigma_def, pos, mo, tmpl_pts, heun)
    match = match_f(K, sigma_data, lm[-1], tmpl_tris, tgt_pts, tgt_tris)
    kp = K.convolve(cp, cp, mom, sigma_def)
    L = -0.5 * match / data_sigma2 - 0.5 * float(np.sum(kp * mom))
    theta_T = grad_f(K, sigma_data, lm[-1], tmpl_tris, tgt_pts, tgt_tris) / (2.0 * data_sigma2)
    theta = adjoint_landmarks(K, sigma_def, pos, mo, lm, theta_T, heun)
    xp, xm = adjoint_diffeo(K, sigma_def, pos, mo, lm, theta, heun)
    g_mom = -xm[0] - kp
    g_cp = -xp[0] - K.grad_alpha(cp, cp, mom, sigma_def, mom)
    return L, g_cp, g_mom, {"match": match, "pos": pos, "mom": mo, "lm": lm, "theta": theta,
                            "xi_pos": xp, "xi_mom": xm}


def registration_multi(K: OracleLib, cp, mom, tmpl_pts, objects, targets, T: int, sigma_def: float,
                       heun: bool = True):
    """registration() for a multi-object template (DeformableMultiObject): the points of every
    object, concatenated in template order, flow together; object i (objects[i] = dict(kind, cells,
    sigma, sigma2, n): data term, template cells, kernel width, data sigma^2, point count) is
    matched to targets[i] = (points, cells). L_data = -0.5 sum_i match_i / sigma2_i
    (DeterministicAtlas.cxx:121-125) and the adjoint is seeded with each object's match gradient
    / (2 sigma2_i) (AbstractAtlas.cxx:585-590)."""
    from . import geometry as G
    pos, mo = shoot(K, sigma_def, cp, mom, T)
    lm = flow_landmarks(K, sigma_def, pos, mo, tmpl_pts, heun)
    matches, theta_T, off = [], [], 0
    for ob, (tp, tc) in zip(objects, targets):
        match_f, grad_f = G.KINDS[ob["kind"]]
        x = lm[-1][off:off + ob["n"]]
        matches.append(match_f(K, ob["sigma"], x, ob["cells"], tp, tc))
        theta_T.append(grad_f(K, ob["sigma"], x, ob["cells"], tp, tc) / (2.0 * ob["sigma2"]))
        off += ob["n"]
    data = 0.0
    for m, ob in zip(matches, objects):
        data -= m / ob["sigma2"]
    data *= 0.5
    kp = K.convolve(cp, cp, mom, sigma_def)
    reg = -0.5 * float(np.sum(kp * mom))
    theta = adjoint_landmarks(K, sigma_def, pos, mo, lm, np.concatenate(theta_T), heun)
    xp, xm = adjoint_diffeo(K, sigma_def, pos, mo, lm, theta, heun)
    g_mom = -xm[0] - kp
    g_cp = -xp[0] - K.grad_alpha(cp, cp, mom, sigma_def, mom)
    return data, reg, g_cp, g_mom, {"matches": matches, "theta": theta, "lm": lm}


def adjoint_landmarks_jumps(K: OracleLib, sigma: float, pos, mom, lm, grads, times, heun: bool = True,
                            t0=0.0, tn=1.0, corrected: bool = False):
    """IntegrateAdjointOfLandmarkPointsEquations with observations (AdjointEquationsIntegrator.cxx:
    59-136, jumps at the observations' time indices `times`, increasing, with match gradients
    `grads`). The reference: with one observation, theta_{T-1} is its gradient; with several,
    theta_{T-1} is the last one's gradient if its index is T - 1, else 0 (:71-87); walking t from
    T - 1 down to 1, the gradient of the observation whose index is t is added to the rate dTheta,
    so it enters multiplied by dt (:104-109); the observation cursor moves back only in the Heun
    branch (:123-128), so the explicit Euler scheme adds at most one observation inside the loop, and
    an observation at index 0 is never added. corrected=True adds every gradient to theta at its own
    index instead (the jump condition of the continuous adjoint, which the registration's adjoint
    discretises the same way)."""
    T = len(pos)
    dt = _dt(T, t0, tn)
    theta = [None] * T
    if corrected:
        theta[T - 1] = np.zeros_like(np.asarray(lm[T - 1], float))
        for g, ti in zip(grads, times):
            if ti == T - 1:
                theta[T - 1] = theta[T - 1] + g
        for t in range(T - 1, 0, -1):
            dth = K.grad_alpha(lm[t], pos[t], mom[t], sigma, theta[t])
            theta[t - 1] = theta[t] + dth * dt
            if heun:
                dth2 = K.grad_alpha(lm[t - 1], pos[t - 1], mom[t - 1], sigma, theta[t - 1])
                theta[t - 1] = theta[t] + (dth + dth2) * (dt * 0.5)
            for g, ti in zip(grads, times):
                if ti == t - 1:
                    theta[t - 1] = theta[t - 1] + g
        return theta
    jumps = len(grads) > 1
    si = len(times) - 1
    if jumps:
        if times[si] == T - 1:
            theta[T - 1] = np.asarray(grads[si], float).copy()
            si = max(si - 1, 0)
        else:
            theta[T - 1] = np.zeros_like(np.asarray(grads[0], float))
    else:
        theta[T - 1] = np.asarray(grads[0], float).copy()
    for t in range(T - 1, 0, -1):
        dth = K.grad_alpha(lm[t], pos[t], mom[t], sigma, theta[t])
        if jumps and t == times[si]:
            dth = dth + grads[si]
        theta[t - 1] = theta[t] + dth * dt
        if heun:
            dth2 = K.grad_alpha(lm[t - 1], pos[t - 1], mom[t - 1], sigma, theta[t - 1])
            if jumps and t == times[si]:
                dth2 = dth2 + grads[si]
                si = max(si - 1, 0)
            theta[t - 1] = theta[t] + (dth + dth2) * (dt * 0.5)
    return theta


def geodesic_regression(K: OracleLib, cp, mom, tmpl, objects, observations, times, T: int, sigma_def: float,
                        t0: float, tn: float, heun: bool = False, corrected: bool = False):
    """Log-likelihood and gradient of the reference's geodesic Regression (Regression.cxx:150-232,
    598-673): the template (objects as in registration_multi) flows along the geodesic of (cp, mom)
    from t0 to tn over T time points; observation s (one (points, cells) per object) is matched to
    the deformed template at time index times[s]. L_data = -sum_s sum_k 0.5 match / sigma2 (:212-214),
    L_reg = -0.5 <K p, p>. The reference's gradient: dL/dp = -xi_mom(0) and dL/dcp = -xi_pos(0)
    only, because AddGradientRegularityTerm (:676-686) takes both gradients by value and its
    subtractions are lost; the landmark adjoint with the reference's jumps; template L2 gradient
    -theta(0). corrected=True: the regularity gradients are subtracted and every observation enters
    the adjoint at its own index; the result then differs from the derivative of the discretised
    log-likelihood only by the O(dt) of the discretised continuous adjoint, as the registration's
    gradient does. Returns (data, reg, g_cp, g_mom, g_tmpl, info)."""
    from . import geometry as G
    pos, mo = shoot(K, sigma_def, cp, mom, T, t0, tn)
    lm = flow_landmarks(K, sigma_def, pos, mo, tmpl, heun, t0, tn)
    data, grads, matches = 0.0, [], []
    for s, targets in enumerate(observations):
        gs, off = [], 0
        for ob, (tp, tc) in zip(objects, targets):
            match_f, grad_f = G.KINDS[ob["kind"]]
            x = lm[times[s]][off:off + ob["n"]]
            r = match_f(K, ob["sigma"], x, ob["cells"], tp, tc)
            matches.append(r)
            data -= 0.5 * r / ob["sigma2"]
            gs.append(grad_f(K, ob["sigma"], x, ob["cells"], tp, tc) / (2.0 * ob["sigma2"]))
            off += ob["n"]
        grads.append(np.concatenate(gs))
    kp = K.convolve(cp, cp, mom, sigma_def)
    reg = 0.0
    for i in range(len(cp)):
        reg -= float(np.dot(kp[i], mom[i]))
    reg *= 0.5
    theta = adjoint_landmarks_jumps(K, sigma_def, pos, mo, lm, grads, times, heun, t0, tn, corrected)
    xp, xm = adjoint_diffeo(K, sigma_def, pos, mo, lm, theta, heun, t0, tn)
    g_cp, g_mom = -xp[0], -xm[0]
    if corrected:
        g_mom = g_mom - kp
        g_cp = g_cp - K.grad_alpha(cp, cp, mom, sigma_def, mom)
    return data, reg, g_cp, g_mom, -theta[0], {"matches": matches, "theta": theta, "lm": lm}
