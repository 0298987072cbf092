// C entry points over the reference's own FP64 kernel layer (test infrastructure only).
//
// This file is compiled together with the unmodified reference sources
// src/support/kernels/ExactKernel.cxx and src/support/kernels/AbstractKernel.cxx (plus the
// Armadillo wrappers they use) into oracle/_ref/libref_exactkernel.so by oracle/build_ref.sh.
// Each function builds ExactKernel<double, d> from row-major arrays, calls exactly one
// reference method and writes the result back row-major. The same symbol names are exported by
// the C restatement in oracle/gauss_oracle.c, so a test can run either library through one
// ctypes binding and compare them.
//
// Return value: 0 on success, -1 when the reference threw (the message is kept for
// oracle_last_error()), -2 for a dimension outside {2, 3}.

#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ExactKernel.h"
#include "P3MKernel.h"

namespace {

thread_local std::string g_last_error;

MatrixType from_rows(const double *p, long rows, long cols) {
  MatrixType M((unsigned)rows, (unsigned)cols, 0.0);
  for (long i = 0; i < rows; ++i)
    for (long j = 0; j < cols; ++j) M((unsigned)i, (unsigned)j) = p[i * cols + j];
  return M;
}

void to_rows(const MatrixType &M, double *out) {
  const unsigned r = M.rows(), c = M.cols();
  for (unsigned i = 0; i < r; ++i)
    for (unsigned j = 0; j < c; ++j) out[(long)i * c + j] = M(i, j);
}

template <unsigned D>
struct Setup {
  ExactKernel<double, D> k;
  Setup(const double *y, const double *w, long ny, int dv, double sigma) {
    k.SetKernelWidth(sigma);
    k.SetSources(from_rows(y, ny, D));
    k.SetWeights(from_rows(w, ny, dv));
  }
};

template <class F>
int guarded(F &&f) {
  try {
    f();
    return 0;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return -1;
  }
}

template <unsigned D>
int convolve_d(int dv, const double *x, long nx, const double *y, const double *w, long ny,
               double sigma, double *out) {
  return guarded([&] {
    Setup<D> s(y, w, ny, dv, sigma);
    to_rows(s.k.Convolve(from_rows(x, nx, D)), out);
  });
}

template <unsigned D>
int grad_alpha_d(int dv, const double *x, long nx, const double *y, const double *w, long ny,
                 double sigma, const double *alpha, double *out) {
  return guarded([&] {
    Setup<D> s(y, w, ny, dv, sigma);
    to_rows(s.k.ConvolveGradient(from_rows(x, nx, D), from_rows(alpha, nx, dv)), out);
  });
}

template <unsigned D>
int grad_varlin_d(int dv, const double *x, long nx, const double *y, const double *w, long ny,
                  double sigma, double *out) {
  return guarded([&] {
    Setup<D> s(y, w, ny, dv, sigma);
    std::vector<MatrixType> g = s.k.ConvolveGradient(from_rows(x, nx, D));
    for (long i = 0; i < nx; ++i) to_rows(g[i], out + i * dv * D);
  });
}

template <unsigned D>
int grad_dim_d(int dv, const double *x, long nx, const double *y, const double *w, long ny,
               double sigma, int dim, double *out) {
  return guarded([&] {
    Setup<D> s(y, w, ny, dv, sigma);
    to_rows(s.k.ConvolveGradient(from_rows(x, nx, D), (unsigned)dim), out);
  });
}

template <unsigned D>
int grad_kdp_d(int dv, const double *x, long nx, const double *y, const double *w, long ny,
               double sigma, int kk, int dp, double *out) {
  return guarded([&] {
    Setup<D> s(y, w, ny, dv, sigma);
    VectorType v = s.k.ConvolveGradient(from_rows(x, nx, D), (unsigned)kk, (unsigned)dp);
    for (unsigned i = 0; i < v.size(); ++i) out[i] = v(i);
  });
}

template <unsigned D>
int hess_full_d(int dv, const double *x, long nx, const double *y, const double *w, long ny,
                double sigma, double *out) {
  return guarded([&] {
    Setup<D> s(y, w, ny, dv, sigma);
    std::vector<std::vector<MatrixType> > h = s.k.ConvolveHessian(from_rows(x, nx, D));
    for (long i = 0; i < nx; ++i)
      for (int kk = 0; kk < dv; ++kk) to_rows(h[i][kk], out + ((i * dv) + kk) * D * D);
  });
}

template <unsigned D>
int hess_rowcol_d(int dv, const double *x, long nx, const double *y, const double *w, long ny,
                  double sigma, int row, int col, double *out) {
  return guarded([&] {
    Setup<D> s(y, w, ny, dv, sigma);
    to_rows(s.k.ConvolveHessian(from_rows(x, nx, D), (unsigned)row, (unsigned)col), out);
  });
}

template <unsigned D>
int hess_kdpdq_d(int dv, const double *x, long nx, const double *y, const double *w, long ny,
                 double sigma, int kk, int dp, int dq, double *out) {
  return guarded([&] {
    Setup<D> s(y, w, ny, dv, sigma);
    VectorType v = s.k.ConvolveHessian(from_rows(x, nx, D), (unsigned)kk, (unsigned)dp, (unsigned)dq);
    for (unsigned i = 0; i < v.size(); ++i) out[i] = v(i);
  });
}

template <unsigned D>
int special_hessian_d(int dv, const double *y, const double *w, long ny, double sigma,
                      const double *xi, double *out) {
  return guarded([&] {
    Setup<D> s(y, w, ny, dv, sigma);
    to_rows(s.k.ConvolveSpecialHessian(from_rows(xi, ny, D)), out);
  });
}

// ExactKernel::ConvolveImageFast (kind 0, out nx x D), ConvolveGradientImageFast(X, image) (kind 1,
// out nx x dv x D) and ConvolveGradientImageFast(X, alpha, image) (kind 2, out nx x D) on an image of
// the given origin, spacing and size (identity direction), through the ITK stand-ins of ref_shim/.
template <unsigned D>
int image_fast_d(int kind, int dv, const double *x, long nx, const double *y, const double *w, long ny,
                 double sigma, const double *alpha, const double *origin, const double *spacing,
                 const long *size, double *out) {
  return guarded([&] {
    Setup<D> s(y, w, ny, dv, sigma);
    auto image = std::make_shared<itk::Image<double, D>>(origin, spacing, size);
    const MatrixType X = from_rows(x, nx, D);
    if (kind == 0) {
      to_rows(s.k.ConvolveImageFast(X, image), out);
    } else if (kind == 1) {
      const std::vector<MatrixType> g = s.k.ConvolveGradientImageFast(X, image);
      for (long i = 0; i < nx; ++i) to_rows(g[(size_t)i], out + i * dv * D);
    } else {
      to_rows(s.k.ConvolveGradientImageFast(X, from_rows(alpha, nx, dv), image), out);
    }
  });
}

// P3MKernel<double, D> (src/support/kernels/P3MKernel.cxx) with its grid parameters: the data domain
// [lo, hi] (the D x 2 matrix SetDataDomain takes), the working spacing ratio and the padding factor,
// through the ITK stand-ins of ref_shim/ (direct DFTs in place of VNL's FFT). kind selects the method:
//  0 Convolve(X)                      out nx x dv
//  1 ConvolveGradient(X)              out nx x dv x D
//  2 ConvolveGradient(X, alpha)       out nx x D
//  3 ConvolveGradient(X, dim = arg0)  out nx x dv
//  4 ConvolveHessian(X)               out nx x dv x D x D
//  5 ConvolveHessian(X, arg0, arg1)   out nx x dv
//  6 ConvolveSpecialHessian(xi = alpha) (AbstractKernel's, over the P3M Hessians; X ignored) out ny x D
//  7 ConvolveGradient(X, arg0, arg1)  out nx (the reference's stub)
//  8 ConvolveHessian(X, arg0, arg1, arg2) out nx (the reference's stub)
template <unsigned D>
int p3m_d(int kind, int dv, const double *x, long nx, const double *y, const double *w, long ny, double sigma,
          const double *alpha, const double *lo, const double *hi, double ratio, double padding, int arg0,
          int arg1, int arg2, double *out) {
  return guarded([&] {
    P3MKernel<double, D> k;
    MatrixType dom(D, 2, 0.0);
    for (unsigned i = 0; i < D; ++i) {
      dom(i, 0) = lo[i];
      dom(i, 1) = hi[i];
    }
    k.SetDataDomain(dom);
    k.SetWorkingSpacingRatio(ratio);
    k.SetPaddingFactor(padding);
    k.SetKernelWidth(sigma);
    k.SetSources(from_rows(y, ny, D));
    k.SetWeights(from_rows(w, ny, dv));
    const MatrixType X = kind == 6 ? MatrixType() : from_rows(x, nx, D);
    switch (kind) {
      case 0: to_rows(k.Convolve(X), out); break;
      case 1: {
        const std::vector<MatrixType> g = k.ConvolveGradient(X);
        for (long i = 0; i < nx; ++i) to_rows(g[(size_t)i], out + i * dv * D);
        break;
      }
      case 2: to_rows(k.ConvolveGradient(X, from_rows(alpha, nx, dv)), out); break;
      case 3: to_rows(k.ConvolveGradient(X, (unsigned)arg0), out); break;
      case 4: {
        const std::vector<std::vector<MatrixType>> h = k.ConvolveHessian(X);
        for (long i = 0; i < nx; ++i)
          for (int c = 0; c < dv; ++c) to_rows(h[(size_t)i][(size_t)c], out + (i * dv + c) * D * D);
        break;
      }
      case 5: to_rows(k.ConvolveHessian(X, (unsigned)arg0, (unsigned)arg1), out); break;
      case 6: to_rows(k.ConvolveSpecialHessian(from_rows(alpha, ny, D)), out); break;
      case 7: {
        const VectorType v = k.ConvolveGradient(X, (unsigned)arg0, (unsigned)arg1);
        for (long i = 0; i < nx; ++i) out[i] = v[(unsigned)i];
        break;
      }
      case 8: {
        const VectorType v = k.ConvolveHessian(X, (unsigned)arg0, (unsigned)arg1, (unsigned)arg2);
        for (long i = 0; i < nx; ++i) out[i] = v[(unsigned)i];
        break;
      }
      default: throw std::runtime_error("unknown P3M method");
    }
  });
}

}  // namespace

#define DISPATCH(fn, ...)                         \
  do {                                            \
    if (d == 2) return fn##_d<2>(__VA_ARGS__);    \
    if (d == 3) return fn##_d<3>(__VA_ARGS__);    \
    return -2;                                    \
  } while (0)

extern "C" {

const char *oracle_last_error(void) { return g_last_error.c_str(); }

int oracle_convolve(int d, int dv, const double *x, long nx, const double *y, const double *w,
                    long ny, double sigma, double *out) {
  DISPATCH(convolve, dv, x, nx, y, w, ny, sigma, out);
}

int oracle_grad_alpha(int d, int dv, const double *x, long nx, const double *y, const double *w,
                      long ny, double sigma, const double *alpha, double *out) {
  DISPATCH(grad_alpha, dv, x, nx, y, w, ny, sigma, alpha, out);
}

int oracle_grad_varlin(int d, int dv, const double *x, long nx, const double *y, const double *w,
                       long ny, double sigma, double *out) {
  DISPATCH(grad_varlin, dv, x, nx, y, w, ny, sigma, out);
}

int oracle_grad_dim(int d, int dv, const double *x, long nx, const double *y, const double *w,
                    long ny, double sigma, int dim, double *out) {
  DISPATCH(grad_dim, dv, x, nx, y, w, ny, sigma, dim, out);
}

int oracle_grad_kdp(int d, int dv, const double *x, long nx, const double *y, const double *w,
                    long ny, double sigma, int k, int dp, double *out) {
  DISPATCH(grad_kdp, dv, x, nx, y, w, ny, sigma, k, dp, out);
}

int oracle_hess_full(int d, int dv, const double *x, long nx, const double *y, const double *w,
                     long ny, double sigma, double *out) {
  DISPATCH(hess_full, dv, x, nx, y, w, ny, sigma, out);
}

int oracle_hess_rowcol(int d, int dv, const double *x, long nx, const double *y, const double *w,
                       long ny, double sigma, int row, int col, double *out) {
  DISPATCH(hess_rowcol, dv, x, nx, y, w, ny, sigma, row, col, out);
}

int oracle_hess_kdpdq(int d, int dv, const double *x, long nx, const double *y, const double *w,
                      long ny, double sigma, int k, int dp, int dq, double *out) {
  DISPATCH(hess_kdpdq, dv, x, nx, y, w, ny, sigma, k, dp, dq, out);
}

int oracle_special_hessian(int d, int dv, const double *y, const double *w, long ny, double sigma,
                           const double *xi, double *out) {
  DISPATCH(special_hessian, dv, y, w, ny, sigma, xi, out);
}

// The image-grid methods (reference library only; the port has no counterpart).
int oracle_ref_image_fast(int d, int kind, int dv, const double *x, long nx, const double *y, const double *w,
                          long ny, double sigma, const double *alpha, const double *origin, const double *spacing,
                          const long *size, double *out) {
  DISPATCH(image_fast, kind, dv, x, nx, y, w, ny, sigma, alpha, origin, spacing, size, out);
}

// P3MKernel's methods (reference library only; see p3m_d for kind and the argument meaning).
int oracle_ref_p3m(int d, int kind, int dv, const double *x, long nx, const double *y, const double *w, long ny,
                   double sigma, const double *alpha, const double *lo, const double *hi, double ratio,
                   double padding, int arg0, int arg1, int arg2, double *out) {
  DISPATCH(p3m, kind, dv, x, nx, y, w, ny, sigma, alpha, lo, hi, ratio, padding, arg0, arg1, arg2, out);
}

}  // extern "C"
