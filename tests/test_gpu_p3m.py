"""GPU particle-mesh kernel (gbk_p3m_*, the reference's P3MKernel with cuFFT) against the reference's
own P3MKernel (golden vectors made by its source compiled on ITK stand-ins,
tests/golden/p3m_reference.npz), against its FP64 restatement (oracle/p3m.py) and against the exact
kernel sums (the reference's P3M tolerance, 8e-2)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gb():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import deformetrica_code_gb300 as g
    return g


@pytest.fixture(scope="module")
def K():
    import oracle
    return oracle.load("port")


@pytest.mark.parametrize("d,sigma", [(2, 0.1), (2, 0.3), (3, 0.3), (3, 0.15)])
def test_p3m_matches_restatement_and_exact(gb, K, d, sigma):
    from oracle import p3m
    from deformetrica_code_gb300 import kernel as KM
    rng = np.random.default_rng(11 + d)
    x, y = rng.random((200, d)), rng.random((250, d))
    w, a = rng.normal(size=(250, 3)), rng.normal(size=(200, 3))
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    v = KM.p3m_convolve(x, y, w, sigma, context=ctx)
    gv = KM.p3m_convolve_gradient(x, y, w, sigma, context=ctx)
    ga = KM.p3m_convolve_gradient_alpha(x, y, w, sigma, a, context=ctx)
    rv, rg = p3m.convolve(x, y, w, sigma), p3m.convolve_gradient(x, y, w, sigma)
    assert np.linalg.norm(v - rv) <= 1e-10 * np.linalg.norm(rv)
    assert np.linalg.norm(gv - rg) <= 1e-10 * np.linalg.norm(rg)
    np.testing.assert_allclose(ga, np.einsum("ikp,ik->ip", gv, a), rtol=1e-12, atol=1e-12 * np.abs(ga).max())
    ve, ge = K.convolve(x, y, w, sigma), K.grad_alpha(x, y, w, sigma, a)
    assert np.linalg.norm(v - ve) <= 8e-2 * np.linalg.norm(ve)
    assert np.linalg.norm(ga - ge) <= 8e-2 * np.linalg.norm(ge)


def test_p3m_domain_and_cache(gb):
    """An explicit data domain equal to the bounding box gives the same sums; a second width after
    the first rebuilds the cached plans and spectra."""
    from oracle import p3m
    from deformetrica_code_gb300 import kernel as KM
    rng = np.random.default_rng(3)
    x, y, w = rng.random((100, 3)), rng.random((120, 3)), rng.normal(size=(120, 2))
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    lo, hi = p3m.domain_of(x, y)
    a = KM.p3m_convolve(x, y, w, 0.3, context=ctx)
    b = KM.p3m_convolve(x, y, w, 0.3, domain=(lo, hi), context=ctx)
    assert np.array_equal(a, b) or np.abs(a - b).max() <= 1e-14 * np.abs(a).max()
    c = KM.p3m_convolve(x, y, w, 0.25, context=ctx)
    assert np.linalg.norm(c - p3m.convolve(x, y, w, 0.25)) <= 1e-10 * np.linalg.norm(c)
    with pytest.raises(ValueError):
        KM.p3m_convolve(x, y, w[:5], 0.3, context=ctx)


@pytest.mark.parametrize("d,sigma", [(2, 0.1), (3, 0.15)])
def test_p3m_f32c_grids(gb, K, d, sigma):
    """GBK_MODE_F32C runs the grids, spectra and transforms in FP32: within 1e-5 (normwise) of the
    FP64 restatement, far inside the method's own error against the exact sums."""
    from oracle import p3m
    from deformetrica_code_gb300 import kernel as KM
    rng = np.random.default_rng(21 + d)
    x, y = rng.random((300, d)), rng.random((280, d))
    w, a = rng.normal(size=(280, 3)), rng.normal(size=(300, 3))
    ctx = gb.Context(mode=gb.GBK_MODE_F32C)
    v = KM.p3m_convolve(x, y, w, sigma, context=ctx)
    gv = KM.p3m_convolve_gradient(x, y, w, sigma, context=ctx)
    ga = KM.p3m_convolve_gradient_alpha(x, y, w, sigma, a, context=ctx)
    rv, rg = p3m.convolve(x, y, w, sigma), p3m.convolve_gradient(x, y, w, sigma)
    assert np.linalg.norm(v - rv) <= 1e-5 * np.linalg.norm(rv)
    assert np.linalg.norm(gv - rg) <= 1e-5 * np.linalg.norm(rg)
    rga = np.einsum("ikp,ik->ip", rg, a)
    assert np.linalg.norm(ga - rga) <= 1e-5 * np.linalg.norm(rga)
    ve = K.convolve(x, y, w, sigma)
    assert np.linalg.norm(v - ve) <= 8e-2 * np.linalg.norm(ve)


def test_p3m_precision_switch(gb):
    """Switching the context's precision between calls rebuilds the cached spectra for that
    precision; switching back reproduces the first result."""
    from oracle import p3m
    from deformetrica_code_gb300 import kernel as KM
    rng = np.random.default_rng(5)
    x, y, w = rng.random((150, 3)), rng.random((160, 3)), rng.normal(size=(160, 3))
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    a = KM.p3m_convolve(x, y, w, 0.2, context=ctx)
    ctx.set_mode(gb.GBK_MODE_F32C)
    b = KM.p3m_convolve(x, y, w, 0.2, context=ctx)
    ctx.set_mode(gb.GBK_MODE_F64)
    c = KM.p3m_convolve(x, y, w, 0.2, context=ctx)
    r = p3m.convolve(x, y, w, 0.2)
    assert np.linalg.norm(a - r) <= 1e-10 * np.linalg.norm(r)
    assert 0 < np.linalg.norm(b - r) <= 1e-5 * np.linalg.norm(r)
    assert np.abs(c - a).max() <= 1e-13 * np.abs(a).max()


@pytest.mark.parametrize("d", [2, 3])
def test_p3m_points_outside_the_domain(gb, d):
    """A data domain smaller than the points: corners that fall off the grid are dropped by the
    splat and the interpolation alike (P3MKernel.cxx:473-593), on the GPU as in the restatement."""
    from oracle import p3m
    from deformetrica_code_gb300 import kernel as KM
    rng = np.random.default_rng(30 + d)
    x, y = rng.uniform(-0.5, 1.5, size=(150, d)), rng.uniform(-0.5, 1.5, size=(170, d))
    w, a = rng.normal(size=(170, 2)), rng.normal(size=(150, 2))
    lo, hi = np.full(d, 0.2), np.full(d, 0.8)
    ctx = gb.Context(mode=gb.GBK_MODE_F64)
    v = KM.p3m_convolve(x, y, w, 0.05, domain=(lo, hi), context=ctx)
    ga = KM.p3m_convolve_gradient_alpha(x, y, w, 0.05, a, domain=(lo, hi), context=ctx)
    rv = p3m.convolve(x, y, w, 0.05, lo, hi)
    rga = p3m.convolve_gradient_alpha(x, y, w, 0.05, a, lo, hi)
    assert np.linalg.norm(v - rv) <= 1e-10 * np.linalg.norm(rv)
    assert np.linalg.norm(ga - rga) <= 1e-10 * np.linalg.norm(rga)
    assert np.count_nonzero(np.all(v == 0, axis=1)) > 0  # targets off the grid get nothing


@pytest.mark.parametrize("d,mode,tol", [(2, "F64", 1e-10), (3, "F64", 1e-10), (3, "F32C", 1e-5)])
def test_p3m_kernel_object_all_overloads(gb, K, d, mode, tol):
    """GB300P3MKernel: every overload of the reference's P3MKernel against the restatement (the two
    stubs return zeros, as the reference's), Hessians within 8e-2 of the exact sums."""
    from oracle import p3m
    rng = np.random.default_rng(40 + d)
    x, y = rng.random((220, d)), rng.random((240, d))
    w, a = rng.normal(size=(240, 2)), rng.normal(size=(220, 2))
    sigma = 0.25
    k = gb.GB300P3MKernel(d, sigma, context=gb.Context(mode=getattr(gb, f"GBK_MODE_{mode}")))
    k.SetSources(y)
    k.SetWeights(w)
    nrm = lambda got, ref: np.linalg.norm(got - ref) / np.linalg.norm(ref)
    assert nrm(k.Convolve(x), p3m.convolve(x, y, w, sigma)) <= tol
    rg = p3m.convolve_gradient(x, y, w, sigma)
    assert nrm(k.ConvolveGradient(x), rg) <= tol
    assert nrm(k.ConvolveGradient(x, a), np.einsum("ikp,ik->ip", rg, a)) <= tol
    for dim in range(d):
        assert nrm(k.ConvolveGradient(x, dim), rg[:, :, dim]) <= tol
    rh = p3m.convolve_hessian(x, y, w, sigma)
    h = k.ConvolveHessian(x)
    assert h.shape == (220, 2, d, d) and nrm(h, rh) <= tol
    assert np.array_equal(h, np.swapaxes(h, 2, 3))
    assert nrm(k.ConvolveHessian(x, d - 1, 0), rh[:, :, 0, d - 1]) <= tol
    he = np.asarray(K.hess_full(x, y, w, sigma)).reshape(rh.shape)
    assert np.linalg.norm(h - he) <= 8e-2 * np.linalg.norm(he)
    assert np.array_equal(k.ConvolveGradient(x, 1, 0), np.zeros(220))
    assert np.array_equal(k.ConvolveHessian(x, 1, 0, d - 1), np.zeros(220))
    with pytest.raises(gb.GBKError):
        k.ConvolveGradient(x, 2, 0)  # weight index out of range, as the reference throws
    with pytest.raises(gb.GBKError):
        k.ConvolveGradient(x, d)  # dimension out of range
    with pytest.raises(gb.GBKError):
        k.ConvolveHessian(x, 0, d)


@pytest.mark.parametrize("d", [2, 3])
def test_p3m_special_hessian(gb, K, d):
    from oracle import p3m
    rng = np.random.default_rng(60 + d)
    y, b, xi = rng.random((150, d)), rng.normal(size=(150, d)), rng.normal(size=(150, d))
    k = gb.GB300P3MKernel(d, 0.3, context=gb.Context(mode=gb.GBK_MODE_F64))
    k.SetSources(y)
    k.SetWeights(b)
    got = k.ConvolveSpecialHessian(xi)
    ref = p3m.special_hessian(y, b, 0.3, xi)
    assert np.linalg.norm(got - ref) <= 1e-10 * np.linalg.norm(ref)
    ex = np.asarray(K.special_hessian(y, b, 0.3, xi)).reshape(ref.shape)
    assert np.linalg.norm(got - ex) <= 8e-2 * np.linalg.norm(ex)


@pytest.mark.parametrize("mode,tol", [("F64", 1e-10), ("F32C", 1e-5)])
@pytest.mark.parametrize("name", ["d2", "d2out", "d3", "d3dv2"])
def test_p3m_matches_the_reference_p3m(gb, name, mode, tol):
    """Every P3MKernel overload on the device against the reference's own outputs (FP64 grids to
    1e-10, FP32 grids to 1e-5 normwise), through the C ABI (kernel.p3m_*) and the kernel object
    (GB300P3MKernel, including the inherited ConvolveSpecialHessian)."""
    from deformetrica_code_gb300 import kernel as KM
    from tests.test_p3m import p3m_case
    c = p3m_case(name)
    x, y, w, sigma = c["x"], c["y"], c["w"], float(c["sigma"])
    d = x.shape[1]
    ctx = gb.Context(mode=getattr(gb, f"GBK_MODE_{mode}"))
    kw = dict(domain=(c["lo"], c["hi"]), spacing_ratio=float(c["ratio"]), padding_factor=float(c["padding"]),
              context=ctx)
    got = {
        "convolve": KM.p3m_convolve(x, y, w, sigma, **kw),
        "gradient": KM.p3m_convolve_gradient(x, y, w, sigma, **kw),
        "gradient_alpha": KM.p3m_convolve_gradient_alpha(x, y, w, sigma, c["alpha"], **kw),
        "gradient_dim": KM.p3m_convolve_gradient_dim(x, y, w, sigma, d - 1, **kw),
        "hessian": KM.p3m_convolve_hessian(x, y, w, sigma, **kw),
        "hessian_rowcol": KM.p3m_convolve_hessian_rowcol(x, y, w, sigma, d - 1, 0, **kw),
    }
    k = gb.GB300P3MKernel(d, sigma, context=ctx, working_spacing_ratio=float(c["ratio"]),
                          padding_factor=float(c["padding"]))
    k.SetSources(c["ys"])
    k.SetWeights(c["beta"])
    k.SetDataDomain(c["ys_lo"], c["ys_hi"])
    got["special_hessian"] = k.ConvolveSpecialHessian(c["xi"])
    for key, val in got.items():
        ref = c[key]
        assert val.shape == ref.shape, key
        assert np.linalg.norm(val - ref) <= tol * np.linalg.norm(ref), (key, np.linalg.norm(val - ref) / np.linalg.norm(ref))
