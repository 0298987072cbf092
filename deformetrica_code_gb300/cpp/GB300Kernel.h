// GB300Kernel.h -- C++ host interface of the GB300 Gaussian kernel sums, over the C ABI of
// include/gbk.h (libgbkernel.so).
//
// gb300::GB300Kernel<PointDim> has the methods, overloads, argument meanings and error behaviour
// of the reference's kernel objects (src/support/kernels/AbstractKernel.h:34-187,
// src/support/kernels/ExactKernel.h:34-194): SetKernelWidth clamps at 1e-10, SetSources /
// SetWeights store the matrices, every Convolve* method returns a new matrix, and shape errors
// throw std::runtime_error (ExactKernel.cxx:58-59, :303-304, :338-344, :455-461). The matrices are
// gb300::Matrix, a row-major double matrix, i.e. the buffers the reference's CUDA path builds with
// vectorise_row_wise() (ArmadilloMatrixWrapper.h:241); a reference build wraps this class in an
// ExactKernel subclass (see the reference binding in GB300ExactKernel.h next to this file).
#pragma once

#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbk.h"

namespace gb300 {

class Matrix {
 public:
  Matrix() : r_(0), c_(0) {}
  Matrix(unsigned r, unsigned c, double v = 0.0) : r_(r), c_(c), d_((size_t)r * c, v) {}
  unsigned rows() const { return r_; }
  unsigned cols() const { return c_; }
  unsigned columns() const { return c_; }
  double &operator()(unsigned i, unsigned j) { return d_[(size_t)i * c_ + j]; }
  const double &operator()(unsigned i, unsigned j) const { return d_[(size_t)i * c_ + j]; }
  double *data() { return d_.data(); }
  const double *data() const { return d_.data(); }

 private:
  unsigned r_, c_;
  std::vector<double> d_;
};

typedef std::vector<double> Vector;

// One library context per thread of use (the reference clones a kernel object per subject
// thread, AbstractAtlas.cxx:218); shared by the kernel objects created on that thread.
class Context {
 public:
  explicit Context(int device = 0, int mode = GBK_MODE_F32C) {
    gbk_ctx *c = nullptr;
    int rc = gbk_create(device, &c);
    if (rc != GBK_OK) throw std::runtime_error(std::string("gbk_create: ") + gbk_last_error(nullptr));
    ctx_.reset(c, gbk_destroy);
    check(gbk_set_mode(c, mode));
  }
  gbk_ctx *get() const { return ctx_.get(); }
  void check(int rc) const {
    if (rc != GBK_OK) throw std::runtime_error(gbk_last_error(ctx_.get()));
  }

 private:
  std::shared_ptr<gbk_ctx> ctx_;
};

template <unsigned PointDim>
class GB300Kernel {
 public:
  explicit GB300Kernel(std::shared_ptr<Context> ctx = std::make_shared<Context>())
      : ctx_(std::move(ctx)) {
    SetKernelWidth(1.0);
    modified_ = false;
  }

  GB300Kernel *Clone() const { return new GB300Kernel(*this); }

  double GetKernelWidth() const { return width_; }
  void SetKernelWidth(double h) {  // AbstractKernel.h:87-93
    if (h < 1e-10) h = 1e-10;
    width_ = h;
    modified_ = true;
  }
  const Matrix &GetSources() const { return Y_; }
  void SetSources(const Matrix &X) {
    if (X.cols() != PointDim) throw std::runtime_error("sources must have PointDim columns");
    Y_ = X;
    modified_ = true;
  }
  const Matrix &GetWeights() const { return W_; }
  void SetWeights(const Matrix &W) {
    W_ = W;
    modified_ = true;
  }
  bool IsModified() const { return modified_; }

  // ExactKernel::Convolve, ExactKernel.cxx:51-74
  Matrix Convolve(const Matrix &X) {
    check_sw();
    Matrix out(X.rows(), W_.cols());
    ctx_->check(gbk_convolve(ctx_->get(), PointDim, W_.cols(), X.data(), X.rows(), Y_.data(), W_.data(),
                             Y_.rows(), width_, out.data()));
    return out;
  }

  // ExactKernel::ConvolveGradient(X) (varlin), ExactKernel.cxx:166-202: one dv x PointDim matrix
  // per target row
  std::vector<Matrix> ConvolveGradient(const Matrix &X) {
    check_sw();
    const unsigned dv = W_.cols();
    std::vector<double> buf((size_t)X.rows() * dv * PointDim);
    ctx_->check(gbk_convolve_gradient(ctx_->get(), PointDim, dv, X.data(), X.rows(), Y_.data(), W_.data(),
                                      Y_.rows(), width_, buf.data()));
    std::vector<Matrix> g(X.rows(), Matrix(dv, PointDim));
    for (unsigned i = 0; i < X.rows(); ++i)
      for (unsigned k = 0; k < dv; ++k)
        for (unsigned l = 0; l < PointDim; ++l) g[i](k, l) = buf[((size_t)i * dv + k) * PointDim + l];
    return g;
  }

  // ExactKernel::ConvolveGradient(X, alpha), ExactKernel.cxx:264-275
  Matrix ConvolveGradient(const Matrix &X, const Matrix &alpha) {
    check_sw();
    if (alpha.rows() != X.rows() || alpha.cols() != W_.cols())
      throw std::runtime_error("alpha must be X.rows() x weights columns");
    Matrix out(X.rows(), PointDim);
    ctx_->check(gbk_convolve_gradient_alpha(ctx_->get(), PointDim, W_.cols(), X.data(), X.rows(), Y_.data(),
                                            W_.data(), Y_.rows(), width_, alpha.data(), out.data()));
    return out;
  }

  // ExactKernel::ConvolveGradient(X, k, dp), ExactKernel.cxx:325-363 (ny results, see gbk.h)
  Vector ConvolveGradient(const Matrix &X, unsigned k, unsigned dp) {
    check_sw();
    Vector out(Y_.rows());
    ctx_->check(gbk_convolve_gradient_kdp(ctx_->get(), PointDim, W_.cols(), X.data(), X.rows(), Y_.data(),
                                          W_.data(), Y_.rows(), width_, (int)k, (int)dp, out.data()));
    return out;
  }

  // ExactKernel::ConvolveGradient(X, dim), ExactKernel.cxx:294-323
  Matrix ConvolveGradient(const Matrix &X, unsigned dim) {
    check_sw();
    Matrix out(X.rows(), W_.cols());
    ctx_->check(gbk_convolve_gradient_dim(ctx_->get(), PointDim, W_.cols(), X.data(), X.rows(), Y_.data(),
                                          W_.data(), Y_.rows(), width_, (int)dim, out.data()));
    return out;
  }

  // ExactKernel::ConvolveHessian(X), ExactKernel.cxx:365-397: H[i][k] (PointDim x PointDim)
  std::vector<std::vector<Matrix>> ConvolveHessian(const Matrix &X) {
    check_sw();
    const unsigned dv = W_.cols(), D = PointDim;
    std::vector<double> buf((size_t)X.rows() * dv * D * D);
    ctx_->check(gbk_convolve_hessian(ctx_->get(), D, dv, X.data(), X.rows(), Y_.data(), W_.data(), Y_.rows(),
                                     width_, buf.data()));
    std::vector<std::vector<Matrix>> h(X.rows(), std::vector<Matrix>(dv, Matrix(D, D)));
    for (unsigned i = 0; i < X.rows(); ++i)
      for (unsigned k = 0; k < dv; ++k)
        for (unsigned a = 0; a < D; ++a)
          for (unsigned b = 0; b < D; ++b) h[i][k](a, b) = buf[(((size_t)i * dv + k) * D + a) * D + b];
    return h;
  }

  // ExactKernel::ConvolveHessian(X, k, dp, dq), ExactKernel.cxx:430-470
  Vector ConvolveHessian(const Matrix &X, unsigned k, unsigned dp, unsigned dq) {
    check_sw();
    Vector out(X.rows());
    ctx_->check(gbk_convolve_hessian_kdpdq(ctx_->get(), PointDim, W_.cols(), X.data(), X.rows(), Y_.data(),
                                           W_.data(), Y_.rows(), width_, (int)k, (int)dp, (int)dq, out.data()));
    return out;
  }

  // ExactKernel::ConvolveHessian(X, row, col), ExactKernel.cxx:399-428
  Matrix ConvolveHessian(const Matrix &X, unsigned row, unsigned col) {
    check_sw();
    Matrix out(X.rows(), W_.cols());
    ctx_->check(gbk_convolve_hessian_rowcol(ctx_->get(), PointDim, W_.cols(), X.data(), X.rows(), Y_.data(),
                                            W_.data(), Y_.rows(), width_, (int)row, (int)col, out.data()));
    return out;
  }

  // AbstractKernel::ConvolveSpecialHessian(xi), AbstractKernel.cxx:22-88
  Matrix ConvolveSpecialHessian(const Matrix &xi) {
    check_sw();
    if (W_.cols() != PointDim) throw std::runtime_error("ConvolveSpecialHessian needs PointDim weight columns");
    if (xi.rows() != Y_.rows()) throw std::runtime_error("Y and Xi count mismatch");
    Matrix out(Y_.rows(), PointDim);
    ctx_->check(gbk_convolve_special_hessian(ctx_->get(), PointDim, Y_.data(), W_.data(), Y_.rows(), width_,
                                             xi.data(), out.data()));
    return out;
  }

 private:
  void check_sw() const {
    if (Y_.rows() != W_.rows()) throw std::runtime_error("Sources and weights count mismatch");
  }

  std::shared_ptr<Context> ctx_;
  Matrix Y_, W_;
  double width_ = 1.0;
  bool modified_ = false;
};

}  // namespace gb300
