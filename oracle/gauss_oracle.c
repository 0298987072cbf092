/*
 * FP64 restatement of the reference's exact Gaussian kernel sums (TEST INFRASTRUCTURE ONLY).
 *
 * This is the oracle: the CUDA library's results are checked against it, and bench.py times it
 * as the CPU baseline. Nothing in the product path may call it. It restates, loop for loop,
 * src/support/kernels/ExactKernel.cxx and src/support/kernels/AbstractKernel.cxx of the
 * reference (Deformetrica 3.0.0), with K(x, y) = exp(-|x - y|^2 / sigma^2)
 * (ExactKernel.h:78-86) and libm exp (src/support/fast_math/MathFunctions.h:19, USE_FAST_MATH
 * off). It exports the same symbols as oracle/ref_driver.cpp (which wraps the reference's own
 * compiled ExactKernel), so tests pin this file against the reference itself.
 *
 * Layout: every matrix is row-major (n rows x c cols), as produced by the reference's
 * vectorise_row_wise() at the CUDA boundary (ArmadilloMatrixWrapper.h:241).
 * Threads: OpenMP over target rows i; every output row is summed by one thread in source order
 * j = 0..ny-1, so results do not depend on the thread count.
 * Return value: 0 ok, -1 argument error (message in oracle_last_error()), -2 bad dimension.
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

static _Thread_local char g_err[256];

const char *oracle_last_error(void) { return g_err; }

static int fail(const char *msg) {
  snprintf(g_err, sizeof g_err, "%s", msg);
  return -1;
}

#define CHECK_D(d) \
  if ((d) != 2 && (d) != 3) return -2

/* exp(-|x_i - y_j|^2 / s2) and the difference x_i - y_j (ExactKernel.h:78-86, :98-110). */
static inline double pair_k(int d, const double *xi, const double *yj, double s2, double *diff) {
  double r2 = 0.0;
  for (int l = 0; l < d; ++l) {
    double t = xi[l] - yj[l];
    diff[l] = t;
    r2 += t * t;
  }
  return exp(-r2 / s2);
}

/* ExactKernel::Convolve, ExactKernel.cxx:51-74: V_i = sum_j K_ij W_j. */
int oracle_convolve(int d, int dv, const double *x, long nx, const double *y, const double *w,
                    long ny, double sigma, double *out) {
  CHECK_D(d);
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nx; ++i) {
    double acc[16] = {0};
    double diff[3];
    for (long j = 0; j < ny; ++j) {
      double k = pair_k(d, x + i * d, y + j * d, s2, diff);
      for (int c = 0; c < dv; ++c) acc[c] += w[j * dv + c] * k;
    }
    for (int c = 0; c < dv; ++c) out[i * dv + c] = acc[c];
  }
  return 0;
}

/* ExactKernel::ConvolveGradient(X) (varlin), ExactKernel.cxx:166-202:
 * G_i(k, l) = sum_j W_jk * dK/dx_l, with dK/dx = (x - y) * (-2 K / sigma^2) (ExactKernel.h:98-110).
 * out is nx x dv x d (row-major per target: [i][k][l]). */
int oracle_grad_varlin(int d, int dv, const double *x, long nx, const double *y, const double *w,
                       long ny, double sigma, double *out) {
  CHECK_D(d);
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nx; ++i) {
    double g_acc[16 * 3] = {0};
    double diff[3];
    for (long j = 0; j < ny; ++j) {
      double k = pair_k(d, x + i * d, y + j * d, s2, diff);
      double f = -2.0 * k / s2;
      for (int c = 0; c < dv; ++c)
        for (int l = 0; l < d; ++l) g_acc[c * d + l] += (diff[l] * f) * w[j * dv + c];
    }
    memcpy(out + i * dv * d, g_acc, sizeof(double) * dv * d);
  }
  return 0;
}

/* ExactKernel::ConvolveGradient(X, alpha), ExactKernel.cxx:264-275: row i = G_i^T alpha_i,
 * i.e. sum_j (alpha_i . W_j) (-2 K_ij / sigma^2)(x_i - y_j). out is nx x d. */
int oracle_grad_alpha(int d, int dv, const double *x, long nx, const double *y, const double *w,
                      long ny, double sigma, const double *alpha, double *out) {
  CHECK_D(d);
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nx; ++i) {
    double g_acc[16 * 3] = {0};
    double diff[3];
    for (long j = 0; j < ny; ++j) {
      double k = pair_k(d, x + i * d, y + j * d, s2, diff);
      double f = -2.0 * k / s2;
      for (int c = 0; c < dv; ++c)
        for (int l = 0; l < d; ++l) g_acc[c * d + l] += (diff[l] * f) * w[j * dv + c];
    }
    for (int l = 0; l < d; ++l) {
      double s = 0.0;
      for (int c = 0; c < dv; ++c) s += g_acc[c * d + l] * alpha[i * dv + c];
      out[i * d + l] = s;
    }
  }
  return 0;
}

/* Term-magnitude sums for condition-aware error measures (test denominators; no reference method).
 * With a_ij = |x_i - y_j|^2 / sigma^2 and weight c_ij = 1 + cond * a_ij (cond = 1: the relative
 * condition number of each term with respect to its inputs, since exp(-a) has condition a; cond = 0:
 * the plain sum of |terms|):
 *   oracle_convolve_mag:   out_ik = sum_j c_ij K_ij |w_jk|
 *   oracle_grad_alpha_mag: out_il = (2 / sigma^2) sum_j c_ij K_ij (sum_k |alpha_ik| |w_jk|) |x_il - y_jl| */
int oracle_convolve_mag(int d, int dv, const double *x, long nx, const double *y, const double *w, long ny,
                        double sigma, int cond, double *out) {
  CHECK_D(d);
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nx; ++i) {
    double acc[16] = {0};
    double diff[3];
    for (long j = 0; j < ny; ++j) {
      double k = pair_k(d, x + i * d, y + j * d, s2, diff);
      double r2 = 0.0;
      for (int l = 0; l < d; ++l) r2 += diff[l] * diff[l];
      const double c = 1.0 + (cond ? r2 / s2 : 0.0);
      for (int q = 0; q < dv; ++q) acc[q] += c * k * fabs(w[j * dv + q]);
    }
    for (int q = 0; q < dv; ++q) out[i * dv + q] = acc[q];
  }
  return 0;
}

int oracle_grad_alpha_mag(int d, int dv, const double *x, long nx, const double *y, const double *w, long ny,
                          double sigma, const double *alpha, int cond, double *out) {
  CHECK_D(d);
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nx; ++i) {
    double acc[3] = {0.0, 0.0, 0.0};
    double diff[3];
    for (long j = 0; j < ny; ++j) {
      double k = pair_k(d, x + i * d, y + j * d, s2, diff);
      double r2 = 0.0, ab = 0.0;
      for (int l = 0; l < d; ++l) r2 += diff[l] * diff[l];
      for (int q = 0; q < dv; ++q) ab += fabs(alpha[i * dv + q]) * fabs(w[j * dv + q]);
      const double c = 1.0 + (cond ? r2 / s2 : 0.0);
      for (int l = 0; l < d; ++l) acc[l] += c * k * ab * fabs(diff[l]);
    }
    for (int l = 0; l < d; ++l) out[i * d + l] = 2.0 * acc[l] / s2;
  }
  return 0;
}

/* ExactKernel::ConvolveGradient(X, dim), ExactKernel.cxx:294-323: sum_j (dK/dx_dim) W_j.
 * out is nx x dv. */
int oracle_grad_dim(int d, int dv, const double *x, long nx, const double *y, const double *w,
                    long ny, double sigma, int dim, double *out) {
  CHECK_D(d);
  if (dim < 0 || dim >= d) return fail("dimension index out of bounds");
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nx; ++i) {
    double acc[16] = {0};
    double diff[3];
    for (long j = 0; j < ny; ++j) {
      double k = pair_k(d, x + i * d, y + j * d, s2, diff);
      double g = diff[dim] * (-2.0 * k / s2);
      for (int c = 0; c < dv; ++c) acc[c] += g * w[j * dv + c];
    }
    for (int c = 0; c < dv; ++c) out[i * dv + c] = acc[c];
  }
  return 0;
}

/* ExactKernel::ConvolveGradient(X, k, dp), ExactKernel.cxx:325-363. Reference quirk kept: the
 * target loop runs over i < ny (the number of SOURCES, :343-347) and the output has ny entries,
 * so X must have at least ny rows (the reference's bounds-checked get_row throws otherwise). */
int oracle_grad_kdp(int d, int dv, const double *x, long nx, const double *y, const double *w,
                    long ny, double sigma, int k, int dp, double *out) {
  CHECK_D(d);
  if (k < 0 || k >= dv) return fail("Invalid weight index");
  if (dp < 0 || dp >= d) return fail("Invalid derivative direction");
  if (nx < ny) return fail("ConvolveGradient(X,k,dp) reads ny rows of X: X has too few rows");
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < ny; ++i) {
    double acc = 0.0;
    double diff[3];
    for (long j = 0; j < ny; ++j) {
      double kk = pair_k(d, x + i * d, y + j * d, s2, diff);
      acc += w[j * dv + k] * (diff[dp] * (-2.0 * kk / s2));
    }
    out[i] = acc;
  }
  return 0;
}

/* Hessian of K(x, y) at x, ExactKernel.h:113-159: K (4 (x-y)(x-y)^T / sigma^4 - 2 I / sigma^2). */
static inline void pair_hess(int d, const double *diff, double k, double s2, double *h) {
  for (int a = 0; a < d; ++a)
    for (int b = 0; b < d; ++b) h[a * d + b] = 4.0 * diff[a] * diff[b] * k / (s2 * s2);
  for (int a = 0; a < d; ++a) h[a * d + a] -= 2.0 * k / s2;
}

/* ExactKernel::ConvolveHessian(X), ExactKernel.cxx:365-397: H_i[k] = sum_j H_ij W_jk.
 * out is nx x dv x d x d. */
int oracle_hess_full(int d, int dv, const double *x, long nx, const double *y, const double *w,
                     long ny, double sigma, double *out) {
  CHECK_D(d);
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nx; ++i) {
    double acc[16 * 9] = {0};
    double diff[3], h[9];
    for (long j = 0; j < ny; ++j) {
      double k = pair_k(d, x + i * d, y + j * d, s2, diff);
      pair_hess(d, diff, k, s2, h);
      for (int c = 0; c < dv; ++c)
        for (int e = 0; e < d * d; ++e) acc[c * d * d + e] += h[e] * w[j * dv + c];
    }
    memcpy(out + i * dv * d * d, acc, sizeof(double) * dv * d * d);
  }
  return 0;
}

/* ExactKernel::ConvolveHessian(X, row, col), ExactKernel.cxx:399-428: sum_j W_j H_ij(row, col).
 * out is nx x dv. */
int oracle_hess_rowcol(int d, int dv, const double *x, long nx, const double *y, const double *w,
                       long ny, double sigma, int row, int col, double *out) {
  CHECK_D(d);
  if (row < 0 || col < 0 || row >= d || col >= d) return fail("Dimension index out of bounds");
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nx; ++i) {
    double acc[16] = {0};
    double diff[3], h[9];
    for (long j = 0; j < ny; ++j) {
      double k = pair_k(d, x + i * d, y + j * d, s2, diff);
      pair_hess(d, diff, k, s2, h);
      for (int c = 0; c < dv; ++c) acc[c] += w[j * dv + c] * h[row * d + col];
    }
    for (int c = 0; c < dv; ++c) out[i * dv + c] = acc[c];
  }
  return 0;
}

/* ExactKernel::ConvolveHessian(X, k, dp, dq), ExactKernel.cxx:430-470: sum_j W_jk H_ij(dp, dq).
 * out has nx entries. */
int oracle_hess_kdpdq(int d, int dv, const double *x, long nx, const double *y, const double *w,
                      long ny, double sigma, int k, int dp, int dq, double *out) {
  CHECK_D(d);
  if (k < 0 || k >= dv) return fail("Invalid weight index");
  if (dp < 0 || dq < 0 || dp >= d || dq >= d) return fail("Invalid derivative direction");
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < nx; ++i) {
    double acc = 0.0;
    double diff[3], h[9];
    for (long j = 0; j < ny; ++j) {
      double kk = pair_k(d, x + i * d, y + j * d, s2, diff);
      pair_hess(d, diff, kk, s2, h);
      acc += w[j * dv + k] * h[dp * d + dq];
    }
    out[i] = acc;
  }
  return 0;
}

/* AbstractKernel::ConvolveSpecialHessian(xi), AbstractKernel.cxx:22-88, over sources Y with
 * weights beta = W (dv must equal d). The reference assembles, from 1 + d(d+1)/2 Hessian sweeps,
 *   dXi4_i = -sum_j (beta_i . beta_j) H_ij xi_i  +  sum_j (beta_i . beta_j) H_ij xi_j
 * (first term :33-43, second term :45-83), i.e. sum_j (beta_i . beta_j) H_ij (xi_j - xi_i) with
 * H_ij the Hessian of K(., y_j) at y_i. This restates that sum directly. out is ny x d. */
int oracle_special_hessian(int d, int dv, const double *y, const double *w, long ny, double sigma,
                           const double *xi, double *out) {
  CHECK_D(d);
  if (dv != d) return fail("ConvolveSpecialHessian needs weights with d columns");
  const double s2 = sigma * sigma;
#pragma omp parallel for schedule(static)
  for (long i = 0; i < ny; ++i) {
    double acc[3] = {0, 0, 0};
    double diff[3], h[9];
    for (long j = 0; j < ny; ++j) {
      double k = pair_k(d, y + i * d, y + j * d, s2, diff);
      pair_hess(d, diff, k, s2, h);
      double bb = 0.0;
      for (int c = 0; c < d; ++c) bb += w[i * d + c] * w[j * d + c];
      for (int a = 0; a < d; ++a) {
        double s = 0.0;
        for (int b = 0; b < d; ++b) s += h[a * d + b] * (xi[j * d + b] - xi[i * d + b]);
        acc[a] += bb * s;
      }
    }
    for (int a = 0; a < d; ++a) out[i * d + a] = acc[a];
  }
  return 0;
}

/* Forward + full adjoint of the scalar L = sum_i alpha_i . V_i with V = Convolve (the work unit
 * of the fused kernel): V_i = sum_j K_ij W_j, gx_i = dL/dx_i (== ConvolveGradient(X, alpha)),
 * gy_j = dL/dy_j = sum_i (alpha_i . W_j)(2 K_ij / sigma^2)(x_i - y_j), gw_j = dL/dW_j =
 * sum_i K_ij alpha_i. The reference has no single method for the source side; by symmetry of K
 * it is ConvolveGradient(Y, W) and Convolve(Y) with sources X and weights alpha, which is how the
 * tests pin this function against the compiled reference. Any output pointer may be NULL. */
int oracle_fwd_adjoint(int d, int dv, const double *x, long nx, const double *y, const double *w,
                       long ny, double sigma, const double *alpha, double *v, double *gx,
                       double *gy, double *gw) {
  CHECK_D(d);
  int rc = 0;
  if (v) rc |= oracle_convolve(d, dv, x, nx, y, w, ny, sigma, v);
  if (gx) rc |= oracle_grad_alpha(d, dv, x, nx, y, w, ny, sigma, alpha, gx);
  if (gw) rc |= oracle_convolve(d, dv, y, ny, x, alpha, nx, sigma, gw);
  if (gy) rc |= oracle_grad_alpha(d, dv, y, ny, x, alpha, nx, sigma, w, gy);
  return rc;
}
