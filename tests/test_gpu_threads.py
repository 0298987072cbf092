"""Concurrent use from several host threads, one context per thread, as the reference's atlas calls
its kernel objects from one thread per subject (AbstractAtlas.cxx:166-205, a kernel object per
thread): every thread's results equal those of the same calls made serially, bit for bit (each
context has its own stream and buffers; the library keeps no other mutable state)."""
import threading

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


def _kernel_work(gb, seed, reps=6):
    rng = np.random.default_rng(seed)
    x, y = rng.random((3000 + 100 * seed, 3)), rng.random((2500 + 50 * seed, 3))
    w, a = rng.normal(size=(y.shape[0], 3)), rng.normal(size=(x.shape[0], 3))
    ctx = gb.Context(mode=gb.GBK_MODE_F32C if seed % 2 else gb.GBK_MODE_F64)
    k = gb.GB300ExactKernel(3, 0.1 + 0.02 * seed, context=ctx)
    k.SetSources(y)
    k.SetWeights(w)
    out = []
    for _ in range(reps):
        out.append(k.Convolve(x))
        out.append(k.ConvolveGradient(x, a))
        out.append(k.ConvolveSpecialHessian(0.5 * y))
    ctx.close()
    return out


def test_kernel_objects_in_threads_match_serial(gb):
    seeds = list(range(6))
    serial = {s: _kernel_work(gb, s) for s in seeds}
    results, errors = {}, []

    def run(s):
        try:
            results[s] = _kernel_work(gb, s)
        except Exception as e:  # reported below
            errors.append(e)

    threads = [threading.Thread(target=run, args=(s,)) for s in seeds]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for s in seeds:
        assert len(results[s]) == len(serial[s])
        for got, ref in zip(results[s], serial[s]):
            assert np.array_equal(got, ref)


def test_registrations_in_threads_match_serial(gb):
    """One registration (graph-replayed iteration) per thread, as the reference's per-subject
    threads."""
    from deformetrica_code_gb300 import meshes as M
    from deformetrica_code_gb300.deformation import Registration
    tp, tf = M.icosphere(2, radius=0.3, center=(0.5, 0.5, 0.5))
    g1 = np.arange(0.25, 0.8, 0.25)
    cp = np.stack(np.meshgrid(g1, g1, g1, indexing="ij"), -1).reshape(-1, 3)

    def work(s):
        rng = np.random.default_rng(40 + s)
        gp = tp + 0.02 * rng.normal(size=tp.shape)
        mom = 0.01 * rng.normal(size=cp.shape)
        ctx = gb.Context()
        reg = Registration(cp.shape[0], tp, tf, gp, tf, T=5, sigma_def=0.25, sigma_data=0.15, data_sigma2=0.01,
                           context=ctx)
        outs = [reg.step(cp, mom) for _ in range(3)]
        reg.close()
        ctx.close()
        return outs

    seeds = list(range(4))
    serial = {s: work(s) for s in seeds}
    results, errors = {}, []

    def run(s):
        try:
            results[s] = work(s)
        except Exception as e:
            errors.append(e)

    threads = [threading.Thread(target=run, args=(s,)) for s in seeds]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=300)
    assert not errors, errors
    for s in seeds:
        for (l1, c1, m1), (l2, c2, m2) in zip(results[s], serial[s]):
            assert np.array_equal(l1, l2) and np.array_equal(c1, c2) and np.array_equal(m1, m2)
