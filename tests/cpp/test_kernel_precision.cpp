// C++ mirror of the reference's TestKernelPrecisionCUDA (tests/unit_tests/kernels/
// TestKernelPrecisionCUDA.cxx:17-203) for gb300::GB300Kernel: the same fixture
// (AbstractTestKernelPrecision: sigma 1.88, X 501 rows, Y 201 rows, std::mt19937(1) re-seeded per
// matrix, entries exp(-gen()/gen.max())), the same operations and the same element-wise criterion
// min(|x-y|/|x|, |x-y|) <= eps. The exact side is the FP64 oracle (oracle/gauss_oracle.c).
// Usage: test_kernel_precision <mode 0=f32c 1=f64> <eps>; exit status 0 when every check passes.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "GB300Kernel.h"

extern "C" {
int oracle_convolve(int, int, const double *, long, const double *, const double *, long, double, double *);
int oracle_grad_alpha(int, int, const double *, long, const double *, const double *, long, double, const double *, double *);
int oracle_grad_varlin(int, int, const double *, long, const double *, const double *, long, double, double *);
int oracle_grad_dim(int, int, const double *, long, const double *, const double *, long, double, int, double *);
int oracle_special_hessian(int, int, const double *, const double *, long, double, const double *, double *);
}

using gb300::Matrix;

static void generate_random_matrix(Matrix &X) {  // AbstractTestKernelPrecision.cxx:21-29
  std::mt19937 gen(1);
  for (unsigned i = 0; i < X.rows(); ++i)
    for (unsigned j = 0; j < X.cols(); ++j) X(i, j) = std::exp(-(double)gen() / (double)(gen.max()));
}

static int failures = 0;
static double eps_tol = 1e-6;

static void compare(const double *exact, const double *gpu, size_t n, const std::string &msg) {
  double worst = 0.0;
  for (size_t i = 0; i < n; ++i) {
    double x = exact[i], y = gpu[i];
    double e = std::min(std::fabs(x - y) / std::fabs(x), std::fabs(x - y));
    if (e > worst) worst = e;
  }
  bool ok = worst <= eps_tol;
  if (!ok) ++failures;
  std::printf("%-40s worst %.3e %s\n", msg.c_str(), worst, ok ? "ok" : "FAIL");
}

template <unsigned D>
static void run(const std::shared_ptr<gb300::Context> &ctx, double w, const Matrix &X, const Matrix &Y,
                const Matrix &W, const Matrix &Z, const std::string &tag) {
  gb300::GB300Kernel<D> k(ctx);
  k.SetKernelWidth(w);
  k.SetSources(Y);
  k.SetWeights(W);
  const int dv = W.cols();
  // Convolve
  Matrix c = k.Convolve(X);
  std::vector<double> ref((size_t)X.rows() * dv * D);
  oracle_convolve(D, dv, X.data(), X.rows(), Y.data(), W.data(), Y.rows(), w, ref.data());
  compare(ref.data(), c.data(), (size_t)X.rows() * dv, tag + " Convolve");
  // ConvolveGradient varlin
  std::vector<Matrix> g = k.ConvolveGradient(X);
  oracle_grad_varlin(D, dv, X.data(), X.rows(), Y.data(), W.data(), Y.rows(), w, ref.data());
  std::vector<double> flat;
  for (auto &m : g) flat.insert(flat.end(), m.data(), m.data() + dv * D);
  compare(ref.data(), flat.data(), flat.size(), tag + " ConvolveGradientVarlin");
  if ((unsigned)dv == D) {
    Matrix ga = k.ConvolveGradient(X, Z);  // ConvolveGradient(X, Z)
    oracle_grad_alpha(D, dv, X.data(), X.rows(), Y.data(), W.data(), Y.rows(), w, Z.data(), ref.data());
    compare(ref.data(), ga.data(), (size_t)X.rows() * D, tag + " ConvolveGradient(X,Z)");
    for (unsigned dim = 0; dim < D; ++dim) {  // ConvolveGradient(Y, int(dim))
      Matrix gd = k.ConvolveGradient(Y, dim);
      oracle_grad_dim(D, dv, Y.data(), Y.rows(), Y.data(), W.data(), Y.rows(), w, (int)dim, ref.data());
      compare(ref.data(), gd.data(), (size_t)Y.rows() * dv, tag + " ConvolveGradient(Y," + std::to_string(dim) + ")");
    }
    Matrix sh = k.ConvolveSpecialHessian(W);
    oracle_special_hessian(D, dv, Y.data(), W.data(), Y.rows(), w, W.data(), ref.data());
    compare(ref.data(), sh.data(), (size_t)Y.rows() * D, tag + " ConvolveSpecialHessian");
  }
}

int main(int argc, char **argv) {
  int mode = argc > 1 ? std::atoi(argv[1]) : GBK_MODE_F32C;
  if (argc > 2) eps_tol = std::atof(argv[2]);
  auto ctx = std::make_shared<gb300::Context>(0, mode);
  const double w = 1.88;
  Matrix X2(501, 2), Y2(201, 2), W2(201, 2), Z2(501, 2), X3(501, 3), Y3(201, 3), W3(201, 3), Z3(501, 3);
  Matrix W4(201, 4), W6(201, 6);
  for (Matrix *m : {&X2, &Y2, &W2, &Z2, &X3, &Y3, &W3, &Z3, &W4, &W6}) generate_random_matrix(*m);
  run<2>(ctx, w, X2, Y2, W2, Z2, "2D W2");
  run<2>(ctx, w, X2, Y2, W4, Z2, "2D W4");
  run<3>(ctx, w, X3, Y3, W3, Z3, "3D W3");
  run<3>(ctx, w, X3, Y3, W6, Z3, "3D W6");
  // error behaviour: sources/weights count mismatch throws std::runtime_error
  gb300::GB300Kernel<3> bad(ctx);
  bad.SetSources(Y3);
  bad.SetWeights(Matrix(200, 3));
  bool threw = false;
  try {
    bad.Convolve(X3);
  } catch (const std::runtime_error &) {
    threw = true;
  }
  if (!threw) ++failures;
  std::printf("mismatch throws: %s\nfailures: %d\n", threw ? "ok" : "FAIL", failures);
  return failures ? 1 : 0;
}
