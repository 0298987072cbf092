"""The C++ host interface: gb300::GB300Kernel (deformetrica_code_gb300/cpp/GB300Kernel.h) driven by
a C++ mirror of the reference's TestKernelPrecisionCUDA on the GPU, and the reference-side binding
(cpp/reference_binding/GB300ExactKernel.h) compiled against the reference's own headers."""
import os
import subprocess

import pytest

from tests.conftest import ROOT

PKG = os.path.join(ROOT, "deformetrica_code_gb300")


def _build_precision_test(tmp):
    import oracle
    oracle.build_port()
    obj = os.path.join(tmp, "gauss_oracle.o")
    subprocess.check_call(["gcc", "-O2", "-fopenmp", "-std=c11", "-c", os.path.join(ROOT, "oracle", "gauss_oracle.c"),
                           "-o", obj])
    exe = os.path.join(tmp, "test_kernel_precision")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(PKG, "cpp"), os.path.join(ROOT, "tests", "cpp", "test_kernel_precision.cpp"),
                           obj, "-L", PKG, "-lgbkernel", "-Wl,-rpath," + PKG, "-fopenmp", "-o", exe])
    return exe


@pytest.mark.gpu
@pytest.mark.parametrize("mode,eps", [(1, 1e-10), (0, 1e-5)])
def test_cpp_kernel_precision(tmp_path, mode, eps):
    """FP64 mode at the reference's double eps_tol (1e-10); compensated FP32 at 1e-5."""
    exe = _build_precision_test(str(tmp_path))
    res = subprocess.run([exe, str(mode), str(eps)], capture_output=True, text=True)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr


def _ref_flags():
    import oracle
    s = os.path.join(oracle.reference_root(), "src", "support")
    arma = os.path.join(ROOT, "oracle", "_ref", "armadillo-7.700.0", "include")
    return ["-std=c++14", "-w", "-DARMA_DONT_USE_WRAPPER", "-DARMA_DONT_USE_LAPACK", "-DARMA_DONT_USE_BLAS",
            "-I" + os.path.join(ROOT, "oracle", "ref_shim"), "-I" + os.path.join(s, "kernels"),
            "-I" + os.path.join(s, "linear_algebra"), "-I" + os.path.join(s, "utilities"),
            "-I" + os.path.join(s, "fast_math"), "-I" + arma, "-I" + os.path.join(ROOT, "include"),
            "-I" + os.path.join(PKG, "cpp", "reference_binding")]


def test_reference_binding_compiles_and_reports_errors(tmp_path):
    """The ExactKernel subclass compiles against the reference headers; linked with the
    reference's ExactKernel objects and libgbkernel.so it raises std::runtime_error (here: no
    GPU) instead of falling back to the CPU."""
    import oracle
    if oracle.build_reference() is None:
        pytest.skip("reference tree not available")
    src = tmp_path / "binding_main.cxx"
    src.write_text(
        '#include "GB300ExactKernel.h"\n#include "GB300P3MKernel.h"\n#include <cstdio>\n'
        "template class GB300ExactKernel<double, 2>;\ntemplate class GB300ExactKernel<double, 3>;\n"
        "template class GB300P3MKernel<double, 2>;\ntemplate class GB300P3MKernel<double, 3>;\n"
        "int main() {\n  GB300ExactKernel<double, 3> k;\n  MatrixType Y(5, 3, 0.5), W(5, 3, 1.0), X(4, 3, 0.25);\n"
        "  k.SetSources(Y); k.SetWeights(W); k.SetKernelWidth(0.3);\n"
        "  try { MatrixType V = k.Convolve(X); std::printf(\"ran %u\\n\", V.rows()); return 0; }\n"
        "  catch (const std::runtime_error &e) { std::printf(\"runtime_error: %s\\n\", e.what()); return 3; }\n}\n")
    objs = [os.path.join(ROOT, "oracle", "_ref", f) for f in
            ("ExactKernel.o", "AbstractKernel.o", "ArmadilloMatrixWrapper.o", "ArmadilloVectorWrapper.o",
             "MatrixListWrapper.o", "SimpleTimer.o")]
    exe = str(tmp_path / "binding_main")
    subprocess.check_call(["g++", *_ref_flags(), str(src), *objs, "-L", PKG, "-lgbkernel", "-Wl,-rpath," + PKG,
                           "-o", exe])
    res = subprocess.run([exe], capture_output=True, text=True)
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        assert res.returncode == 0 and "ran 4" in res.stdout
    else:
        assert res.returncode == 3 and "runtime_error" in res.stdout, res.stdout + res.stderr


def _build_binding_test(tmp):
    import oracle
    oracle.build_port()
    obj = os.path.join(tmp, "gauss_oracle.o")
    subprocess.check_call(["gcc", "-O2", "-fopenmp", "-std=c11", "-c", os.path.join(ROOT, "oracle", "gauss_oracle.c"),
                           "-o", obj])
    exe = os.path.join(tmp, "test_binding")
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "tests", "cpp", "binding_standin"),
                           "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(PKG, "cpp", "reference_binding"),
                           os.path.join(ROOT, "tests", "cpp", "test_binding.cpp"), obj, "-L", PKG, "-lgbkernel",
                           "-Wl,-rpath," + PKG, "-fopenmp", "-o", exe])
    return exe


@pytest.mark.gpu
@pytest.mark.parametrize("mode,eps,eps_cancel", [("f64", 1e-10, 1e-10), ("f32c", 1e-5, 1e-4)])
def test_reference_binding_runs_on_the_gpu(tmp_path, mode, eps, eps_cancel):
    """GB300ExactKernel (the reference binding) on the GPU, over a stand-in of the reference's base
    class: every override against the FP64 oracle (the reference's element-wise criterion; in FP32C
    the Hessian-type outputs, cancellations of larger terms, at 1e-4), sources uploaded once per
    modification, the image methods equal to direct C-ABI calls, shape errors thrown."""
    exe = _build_binding_test(str(tmp_path))
    env = dict(os.environ, GBK_MODE=mode)
    res = subprocess.run([exe, str(eps), str(eps_cancel)], capture_output=True, text=True, env=env, timeout=300)
    print(res.stdout)
    assert res.returncode == 0, res.stdout + res.stderr


def test_reference_binding_compiles_against_the_standin():
    """The same program compiles on any host (no GPU needed to build it)."""
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        assert os.path.exists(_build_binding_test(tmp))
