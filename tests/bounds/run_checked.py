"""Runs a battery of kernel sums through whichever build of the library $GBK_LIBRARY names and saves
the outputs (npz at argv[1]); after every call the context is synchronised, so an index check that
failed in a bounds-checked build raises GBKError (GBK_ERR_BOUNDS). Used by
tests/test_gpu_bounds_check.py; needs a GPU."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
import deformetrica_code_gb300 as g  # noqa: E402
from deformetrica_code_gb300 import kernel as KM  # noqa: E402
from deformetrica_code_gb300.deformation import Deformation, Registration  # noqa: E402


def mixture(rng, n, d, lo=0.15, hi=0.85):
    means = rng.uniform(lo, hi, (8, d))
    return np.ascontiguousarray(means[rng.integers(0, 8, n)] + 0.05 * rng.standard_normal((n, d)))


def main(path):
    rng = np.random.default_rng(123)
    out = {}
    ctx = g.Context()
    orders = {"auto": g.GBK_ORDER_AUTO, "off": g.GBK_ORDER_OFF, "two_float": g.GBK_ORDER_TWO_FLOAT,
              "spatial": g.GBK_ORDER_SPATIAL, "noprune": g.GBK_ORDER_SPATIAL_NOPRUNE}
    # sizes for the warp-split, small and default shapes; ragged counts
    for d in (2, 3):
        for nx, ny in ((97, 1001), (1000, 10242), (4099, 5003), (70001, 65537)):
            X, Y = mixture(rng, nx, d), mixture(rng, ny, d)
            W, A = rng.standard_normal((ny, d)), rng.standard_normal((nx, d))
            for mode_name, mode in (("f32c", g.GBK_MODE_F32C), ("f64", g.GBK_MODE_F64)):
                if mode == g.GBK_MODE_F64 and nx * ny > 1e8:
                    continue
                ctx.set_mode(mode)
                for oname, order in orders.items():
                    if oname == "noprune" and nx * ny > 1e9:
                        continue
                    ctx.set_order(order)
                    for split in ((0, 3) if nx * ny < 1e9 else (0,)):
                        ctx.set_split(split)
                        k = g.GB300ExactKernel(d, 0.05, context=ctx)
                        k.SetSources(Y)
                        k.SetWeights(W)
                        key = f"d{d}_{nx}x{ny}_{mode_name}_{oname}_s{split}"
                        res = list(k.ForwardAdjoint(X, A))
                        ctx.synchronize()
                        if nx * ny < 1e8:
                            res += [k.ConvolveGradient(X), k.ConvolveGradient(X, d - 1), k.ConvolveHessian(X),
                                    k.ConvolveHessian(X, 0, d - 1)]
                            ctx.synchronize()
                            ks = g.GB300ExactKernel(d, 0.05, context=ctx)
                            ks.SetSources(Y[:nx])
                            ks.SetWeights(W[:nx] if ny >= nx else A[:nx])
                            res.append(ks.ConvolveSpecialHessian(A[:nx] if ny >= nx else A))
                            ctx.synchronize()
                        for i, r in enumerate(res):
                            out[f"{key}_{i}"] = np.asarray(r)
    ctx.set_split(0)
    ctx.set_order(g.GBK_ORDER_AUTO)
    ctx.set_mode(g.GBK_MODE_F32C)
    # the control-point adjoint update and a registration step (graph capture and replay)
    for d in (2, 3):
        cp = rng.uniform(0.2, 0.8, (300, d))
        mom, xp, xm = (rng.standard_normal((300, d)) for _ in range(3))
        lm, th = rng.uniform(0.1, 0.9, (911, d)), rng.standard_normal((911, d))
        df = Deformation(d, 0.2, 2, context=ctx)
        for i, r in enumerate(df.compute_update_at(cp, mom, xp, xm, lm, th)):
            out[f"adj_d{d}_{i}"] = np.asarray(r)
        ctx.synchronize()
    from deformetrica_code_gb300 import meshes as M
    tp, tf = M.icosphere(3, 0.4)
    gp = M.sine_bump(tp, tf, 0.05, 4.0)
    g1 = np.arange(0.1, 1.0, 0.2)
    cp = np.stack(np.meshgrid(g1, g1, g1, indexing="ij"), -1).reshape(-1, 3)
    mom = 0.01 * rng.standard_normal(cp.shape)
    reg = Registration(cp.shape[0], tp, tf, gp, tf, T=6, sigma_def=0.2, sigma_data=0.1, data_sigma2=0.01,
                       context=ctx)
    for it in range(3):
        ll, gc, gm = reg.step(cp, mom)
        ctx.synchronize()
    out["reg_ll"], out["reg_gc"], out["reg_gm"] = ll, gc, gm
    # particle-mesh kernel
    x, y, w = rng.random((5000, 3)), rng.random((6000, 3)), rng.standard_normal((6000, 3))
    out["p3m"] = KM.p3m_convolve(x, y, w, 0.2, context=ctx)
    ctx.synchronize()
    np.savez(path, **out)


if __name__ == "__main__":
    main(sys.argv[1])
