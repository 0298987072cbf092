// Test-only stand-in for the reference's kernel base classes (src/support/kernels/AbstractKernel.h,
// ExactKernel.h) and matrix types (src/support/linear_algebra/LinearAlgebra.h), so the reference
// binding GB300ExactKernel.h compiles and runs where the reference tree is absent (the GPU machine). It
// declares only what the binding uses, with the reference's names and meanings: row-major-vectorising
// matrices, the kernel width clamp, and the m_Modified flag that SetSources / SetWeights /
// SetKernelWidth set. Every convolution method of the stand-in base throws: the binding overrides
// all of them. The parity of the binding itself is checked against the FP64 oracle by
// tests/cpp/test_binding.cpp; where the reference tree exists, tests/test_cpp_dropin.py also
// compiles the binding against the reference's own headers and objects.
#pragma once

#include <memory>
#include <stdexcept>
#include <vector>

#include "itkImage.h"  // the oracle's ITK stand-ins (identity-direction images)

class VectorType {
 public:
  VectorType() {}
  explicit VectorType(const std::vector<double> &v) : d_(v) {}
  unsigned size() const { return (unsigned)d_.size(); }
  double &operator()(unsigned i) { return d_[i]; }
  double operator()(unsigned i) const { return d_[i]; }
  double *memptr() { return d_.data(); }
  const double *memptr() const { return d_.data(); }

 private:
  std::vector<double> d_;
};

class MatrixType {
 public:
  MatrixType() : r_(0), c_(0) {}
  MatrixType(unsigned r, unsigned c, double v = 0.0) : r_(r), c_(c), d_((size_t)r * c, v) {}
  unsigned rows() const { return r_; }
  unsigned cols() const { return c_; }
  unsigned columns() const { return c_; }
  double &operator()(unsigned i, unsigned j) { return d_[(size_t)i * c_ + j]; }
  double operator()(unsigned i, unsigned j) const { return d_[(size_t)i * c_ + j]; }
  VectorType vectorise_row_wise() const { return VectorType(d_); }  // storage is row-major already

 private:
  unsigned r_, c_;
  std::vector<double> d_;
};

template <class ScalarType, unsigned int PointDim>
class ExactKernel {
 public:
  typedef itk::Image<ScalarType, PointDim> ImageType;
  typedef typename ImageType::Pointer ImageTypePointer;

  ExactKernel() : m_KernelWidth(1.0), m_Modified(false) {}
  ExactKernel(const ExactKernel &o) = default;
  ExactKernel(const MatrixType &X, double h) : m_Sources(X), m_Modified(true) { SetKernelWidth(h); }
  ExactKernel(const MatrixType &X, const MatrixType &W, double h) : m_Sources(X), m_Weights(W), m_Modified(true) {
    SetKernelWidth(h);
  }
  virtual ~ExactKernel() {}
  virtual ExactKernel *Clone() const = 0;

  double GetKernelWidth() const { return m_KernelWidth; }
  virtual void SetKernelWidth(double h) {  // AbstractKernel.h:85-91
    m_KernelWidth = h < 1e-10 ? 1e-10 : h;
    m_Modified = true;
  }
  MatrixType &GetSources() { return m_Sources; }
  void SetSources(const MatrixType &X) {
    m_Sources = X;
    m_Modified = true;
  }
  MatrixType &GetWeights() { return m_Weights; }
  void SetWeights(const MatrixType &W) {
    m_Weights = W;
    m_Modified = true;
  }
  bool IsModified() const { return m_Modified; }
  void SetModified() { m_Modified = true; }
  void UnsetModified() { m_Modified = false; }

  virtual MatrixType Convolve(const MatrixType &) { throw std::runtime_error("stand-in base"); }
  virtual std::vector<MatrixType> ConvolveGradient(const MatrixType &) { throw std::runtime_error("stand-in base"); }
  virtual MatrixType ConvolveGradient(const MatrixType &, const MatrixType &) { throw std::runtime_error("stand-in base"); }
  virtual VectorType ConvolveGradient(const MatrixType &, unsigned, unsigned) { throw std::runtime_error("stand-in base"); }
  virtual MatrixType ConvolveGradient(const MatrixType &, unsigned) { throw std::runtime_error("stand-in base"); }
  virtual std::vector<std::vector<MatrixType> > ConvolveHessian(const MatrixType &) {
    throw std::runtime_error("stand-in base");
  }
  virtual VectorType ConvolveHessian(const MatrixType &, unsigned, unsigned, unsigned) {
    throw std::runtime_error("stand-in base");
  }
  virtual MatrixType ConvolveHessian(const MatrixType &, unsigned, unsigned) { throw std::runtime_error("stand-in base"); }
  virtual MatrixType ConvolveSpecialHessian(const MatrixType &) { throw std::runtime_error("stand-in base"); }
  virtual MatrixType ConvolveImageFast(const MatrixType &, const ImageTypePointer) {
    throw std::runtime_error("stand-in base");
  }
  virtual std::vector<MatrixType> ConvolveGradientImageFast(const MatrixType &, const ImageTypePointer) {
    throw std::runtime_error("stand-in base");
  }
  virtual MatrixType ConvolveGradientImageFast(const MatrixType &, const MatrixType &, const ImageTypePointer) {
    throw std::runtime_error("stand-in base");
  }

 protected:
  MatrixType m_Sources, m_Weights;
  double m_KernelWidth;
  bool m_Modified;
};
