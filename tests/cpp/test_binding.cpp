// Runs the reference binding GB300ExactKernel (deformetrica_code_gb300/cpp/reference_binding/
// GB300ExactKernel.h) on the GPU: every overridden method against the FP64 oracle
// (oracle/gauss_oracle.c) with the reference's element-wise criterion min(|x-y|/|x|, |x-y|) <= eps,
// the image methods against direct C-ABI calls, the device copies of the sources uploaded once per
// modification, and the shape errors thrown as std::runtime_error. Built against the stand-in base
// of tests/cpp/binding_standin where the reference tree is absent.
// Usage: test_binding <eps> [<eps_cancel>]; eps_cancel (default eps) bounds the outputs whose elements
// are cancellations of larger terms (the Hessians' 4/sigma^4 S - 2/sigma^2 C, the special Hessian's
// xi_j - xi_i), where an element-wise relative criterion measures the cancellation, not the arithmetic.
// The precision comes from GBK_MODE as in the binding. Exit 0 on success.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "GB300ExactKernel.h"

extern "C" {
int oracle_convolve(int, int, const double *, long, const double *, const double *, long, double, double *);
int oracle_grad_alpha(int, int, const double *, long, const double *, const double *, long, double, const double *,
                      double *);
int oracle_grad_varlin(int, int, const double *, long, const double *, const double *, long, double, double *);
int oracle_grad_dim(int, int, const double *, long, const double *, const double *, long, double, int, double *);
int oracle_grad_kdp(int, int, const double *, long, const double *, const double *, long, double, int, int, double *);
int oracle_hess_full(int, int, const double *, long, const double *, const double *, long, double, double *);
int oracle_hess_rowcol(int, int, const double *, long, const double *, const double *, long, double, int, int,
                       double *);
int oracle_hess_kdpdq(int, int, const double *, long, const double *, const double *, long, double, int, int, int,
                      double *);
int oracle_special_hessian(int, int, const double *, const double *, long, double, const double *, double *);
}

static int failures = 0;
static double eps_tol = 1e-10;
static double eps_cancel = 1e-10;

static void check(bool ok, const std::string &msg) {
  if (!ok) ++failures;
  std::printf("%-52s %s\n", msg.c_str(), ok ? "ok" : "FAIL");
}

static void compare(const std::vector<double> &exact, const std::vector<double> &got, const std::string &msg,
                    bool cancel = false) {
  double worst = 0.0;
  bool same_size = exact.size() == got.size();
  for (size_t i = 0; same_size && i < exact.size(); ++i) {
    const double x = exact[i], y = got[i], e = std::min(std::fabs(x - y) / std::fabs(x), std::fabs(x - y));
    worst = std::max(worst, e);
  }
  const bool ok = same_size && worst <= (cancel ? eps_cancel : eps_tol);
  if (!ok) ++failures;
  std::printf("%-52s worst %.3e %s\n", msg.c_str(), worst, ok ? "ok" : "FAIL");
}

static MatrixType random_matrix(unsigned r, unsigned c, std::mt19937 &gen, double lo, double hi) {
  std::uniform_real_distribution<double> u(lo, hi);
  MatrixType M(r, c);
  for (unsigned i = 0; i < r; ++i)
    for (unsigned j = 0; j < c; ++j) M(i, j) = u(gen);
  return M;
}

static std::vector<double> rows_of(const MatrixType &M) {
  std::vector<double> v;
  for (unsigned i = 0; i < M.rows(); ++i)
    for (unsigned j = 0; j < M.cols(); ++j) v.push_back(M(i, j));
  return v;
}

template <unsigned D>
static void run(unsigned dv) {
  std::mt19937 gen(7 + D + dv);
  const unsigned nx = 301, ny = 257;
  const double sigma = 0.35;
  const MatrixType X = random_matrix(nx, D, gen, 0.0, 1.0), Y = random_matrix(ny, D, gen, 0.0, 1.0);
  const MatrixType W = random_matrix(ny, dv, gen, -1.0, 1.0), A = random_matrix(nx, dv, gen, -1.0, 1.0);
  const MatrixType Xi = random_matrix(ny, D, gen, -1.0, 1.0), Wd = random_matrix(ny, D, gen, -1.0, 1.0);
  const std::vector<double> x = rows_of(X), y = rows_of(Y), w = rows_of(W), a = rows_of(A), xi = rows_of(Xi),
                            wd = rows_of(Wd);
  const std::string tag = "d=" + std::to_string(D) + " dv=" + std::to_string(dv) + " ";
  GB300ExactKernel<double, D> k;
  k.SetKernelWidth(sigma);
  k.SetSources(Y);
  k.SetWeights(W);
  std::vector<double> ref;

  ref.assign((size_t)nx * dv, 0.0);
  oracle_convolve(D, dv, x.data(), nx, y.data(), w.data(), ny, sigma, ref.data());
  compare(ref, rows_of(k.Convolve(X)), tag + "Convolve");

  ref.assign((size_t)nx * dv * D, 0.0);
  oracle_grad_varlin(D, dv, x.data(), nx, y.data(), w.data(), ny, sigma, ref.data());
  std::vector<double> got;
  for (const MatrixType &G : k.ConvolveGradient(X)) {
    const std::vector<double> g = rows_of(G);
    got.insert(got.end(), g.begin(), g.end());
  }
  compare(ref, got, tag + "ConvolveGradient(X)");

  ref.assign((size_t)nx * D, 0.0);
  oracle_grad_alpha(D, dv, x.data(), nx, y.data(), w.data(), ny, sigma, a.data(), ref.data());
  compare(ref, rows_of(k.ConvolveGradient(X, A)), tag + "ConvolveGradient(X, alpha)");

  ref.assign((size_t)nx * dv, 0.0);
  oracle_grad_dim(D, dv, x.data(), nx, y.data(), w.data(), ny, sigma, D - 1, ref.data());
  compare(ref, rows_of(k.ConvolveGradient(X, D - 1)), tag + "ConvolveGradient(X, dim)");

  ref.assign(ny, 0.0);
  oracle_grad_kdp(D, dv, x.data(), nx, y.data(), w.data(), ny, sigma, dv - 1, 0, ref.data());
  const VectorType kdp = k.ConvolveGradient(X, dv - 1, 0);
  compare(ref, std::vector<double>(kdp.memptr(), kdp.memptr() + kdp.size()), tag + "ConvolveGradient(X, k, dp)");

  ref.assign((size_t)nx * dv * D * D, 0.0);
  oracle_hess_full(D, dv, x.data(), nx, y.data(), w.data(), ny, sigma, ref.data());
  got.clear();
  for (const auto &Hi : k.ConvolveHessian(X))
    for (const MatrixType &H : Hi) {
      const std::vector<double> h = rows_of(H);
      got.insert(got.end(), h.begin(), h.end());
    }
  compare(ref, got, tag + "ConvolveHessian(X)", true);

  ref.assign((size_t)nx * dv, 0.0);
  oracle_hess_rowcol(D, dv, x.data(), nx, y.data(), w.data(), ny, sigma, 0, D - 1, ref.data());
  compare(ref, rows_of(k.ConvolveHessian(X, 0u, D - 1)), tag + "ConvolveHessian(X, row, col)", true);

  ref.assign(nx, 0.0);
  oracle_hess_kdpdq(D, dv, x.data(), nx, y.data(), w.data(), ny, sigma, 0, D - 1, 0, ref.data());
  const VectorType kdpdq = k.ConvolveHessian(X, 0u, D - 1, 0u);
  compare(ref, std::vector<double>(kdpdq.memptr(), kdpdq.memptr() + kdpdq.size()), tag + "ConvolveHessian(X, k, dp, dq)", true);

  check(k.SourceUploads() == 1, tag + "sources uploaded once for 8 calls");
  k.SetWeights(Wd);  // marks the object modified: the next call uploads again
  ref.assign((size_t)ny * D, 0.0);
  oracle_special_hessian(D, D, y.data(), wd.data(), ny, sigma, xi.data(), ref.data());
  compare(ref, rows_of(k.ConvolveSpecialHessian(Xi)), tag + "ConvolveSpecialHessian(xi)", true);
  check(k.SourceUploads() == 2, tag + "uploaded again after SetWeights");
  ref.assign((size_t)nx * D, 0.0);
  oracle_convolve(D, D, x.data(), nx, y.data(), wd.data(), ny, sigma, ref.data());
  compare(ref, rows_of(k.Convolve(X)), tag + "Convolve with the new weights");
  check(k.SourceUploads() == 2, tag + "no upload without a change");

  // image methods: the binding against the direct C-ABI calls on the same image. The window is
  // int(6 sigma) pixels from the index of y - 3 sigma, so sigma is in pixels (spacing ~1) and the
  // control points lie over the image.
  const long n[3] = {11, 9, 7};
  const double o[3] = {0.0, 0.5, -0.5}, s[3] = {1.0, 1.1, 0.9};
  const double sig_img = 1.5;
  long npix = 1;
  for (unsigned i = 0; i < D; ++i) npix *= n[i];
  auto image = std::make_shared<itk::Image<double, D>>(o, s, n);
  std::vector<double> pts((size_t)npix * D);
  gb300_binding::check(gbk_image_points(gb300_binding::thread_context(), D, o, s, n, pts.data()));
  MatrixType P(npix, D), Yi(ny, D);
  for (long i = 0; i < npix; ++i)
    for (unsigned l = 0; l < D; ++l) P(i, l) = pts[(size_t)i * D + l];
  for (unsigned j = 0; j < ny; ++j)
    for (unsigned l = 0; l < D; ++l) Yi(j, l) = o[l] + Y(j, l) * s[l] * (n[l] - 1);
  const std::vector<double> yi = rows_of(Yi);
  const MatrixType Ai = random_matrix(npix, D, gen, -1.0, 1.0);
  const std::vector<double> ai = rows_of(Ai);
  GB300ExactKernel<double, D> ki(Yi, Wd, sig_img);
  std::vector<double> direct((size_t)npix * D);
  gb300_binding::check(gbk_convolve_image_fast(gb300_binding::thread_context(), D, pts.data(), npix, yi.data(),
                                               wd.data(), ny, sig_img, o, s, n, direct.data()));
  compare(direct, rows_of(ki.ConvolveImageFast(P, image)), tag + "ConvolveImageFast");
  direct.assign((size_t)npix * D, 0.0);
  gb300_binding::check(gbk_convolve_gradient_image_fast_alpha(gb300_binding::thread_context(), D, D, pts.data(), npix,
                                                              yi.data(), wd.data(), ny, sig_img, ai.data(), o, s, n,
                                                              direct.data()));
  compare(direct, rows_of(ki.ConvolveGradientImageFast(P, Ai, image)), tag + "ConvolveGradientImageFast(X, alpha)");
  direct.assign((size_t)npix * D * D, 0.0);
  gb300_binding::check(gbk_convolve_gradient_image_fast(gb300_binding::thread_context(), D, D, pts.data(), npix,
                                                        yi.data(), wd.data(), ny, sig_img, o, s, n, direct.data()));
  got.clear();
  for (const MatrixType &G : ki.ConvolveGradientImageFast(P, image)) {
    const std::vector<double> g = rows_of(G);
    got.insert(got.end(), g.begin(), g.end());
  }
  compare(direct, got, tag + "ConvolveGradientImageFast(X)");

  // shape errors are std::runtime_error, as the reference throws them
  GB300ExactKernel<double, D> bad;
  bad.SetSources(Y);
  bad.SetWeights(MatrixType(ny - 1, dv));
  bool threw = false;
  try {
    bad.Convolve(X);
  } catch (const std::runtime_error &) {
    threw = true;
  }
  check(threw, tag + "count mismatch throws");
}

int main(int argc, char **argv) {
  if (argc > 1) eps_tol = eps_cancel = std::atof(argv[1]);
  if (argc > 2) eps_cancel = std::atof(argv[2]);
  try {
    run<3>(3);
    run<3>(6);
    run<2>(2);
    run<2>(4);
  } catch (const std::exception &e) {
    std::printf("exception: %s\n", e.what());
    return 2;
  }
  std::printf("%d failure(s)\n", failures);
  return failures ? 1 : 0;
}
