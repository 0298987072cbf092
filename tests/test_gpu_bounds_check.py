"""GPU: the bounds-checked build of the library (-DGBK_BOUNDS_CHECK=1, libgbkernel_checked.so: every
target and source index the kernel sums compute is checked against its array before use; a failure
is clamped and reported as GBK_ERR_BOUNDS by gbk_synchronize). A battery of kernel sums over the
warp-split, small, default and bulk-staged shapes, every order (caller, two-float, spatial with and
without pruning), forced source splits, both precisions, ragged sizes, the adjoint update, a
registration step (graph capture and replay) and the particle-mesh kernel runs through the checked
build with a synchronisation after every call (tests/bounds/run_checked.py): no index check may
fail, and the results must equal the default build's to rounding (the checks only read indices, but
the compiler may contract the FP64 output scaling of a few kernels differently in the two builds;
the particle-mesh splat's atomics add in any order).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RUNNER = os.path.join(ROOT, "tests", "bounds", "run_checked.py")


def test_checked_build_reports_no_out_of_bounds_index(tmp_path):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    import importlib.util
    spec = importlib.util.spec_from_file_location("_gbk_build", os.path.join(ROOT, "deformetrica_code_gb300", "build.py"))
    build = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(build)
    checked = build.build(bounds_check=True)
    default = build.build()
    results = {}
    for name, lib in (("checked", checked), ("default", default)):
        env = dict(os.environ, GBK_LIBRARY=lib)
        out = tmp_path / f"{name}.npz"
        res = subprocess.run([sys.executable, RUNNER, str(out)], env=env, capture_output=True, text=True, timeout=900)
        assert res.returncode == 0, f"{name} build:\n{res.stdout[-2000:]}\n{res.stderr[-4000:]}"
        results[name] = np.load(out)
    a, b = results["checked"], results["default"]
    assert sorted(a.files) == sorted(b.files) and len(a.files) > 100
    same = 0
    for key in a.files:
        x, y = a[key], b[key]
        assert x.shape == y.shape and np.array_equal(np.isnan(x), np.isnan(y)), key
        x, y = np.nan_to_num(x), np.nan_to_num(y)
        tol = 1e-6 if key.startswith("p3m") else 1e-12  # the splat's FP32 atomics add in any order
        assert np.linalg.norm(x - y) <= tol * np.linalg.norm(y), key
        same += np.array_equal(x, y)
    assert same >= 0.9 * len(a.files)  # nearly all bitwise equal
