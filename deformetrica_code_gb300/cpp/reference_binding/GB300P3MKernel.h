// GB300P3MKernel.h -- the particle-mesh kernel a Deformetrica build can use in place of
// src/support/kernels/P3MKernel.h: the same base (ExactKernel, as P3MKernel derives from it), the
// same grid settings (SetDataDomain: PointDim x 2, minimum and maximum per axis;
// SetWorkingSpacingRatio; SetPaddingFactor) and every convolution overload of P3MKernel
// (P3MKernel.cxx:1245-1729) as one call into the C ABI of include/gbk.h. ConvolveSpecialHessian is
// inherited from AbstractKernel (AbstractKernel.cxx:22-88) and composes these overloads, as it does
// for the reference's P3MKernel. Failures throw std::runtime_error with the library's message.
#pragma once

#include "GB300ExactKernel.h"

template <class ScalarType, unsigned int PointDim>
class GB300P3MKernel : public ExactKernel<ScalarType, PointDim> {
 public:
  typedef ExactKernel<ScalarType, PointDim> Superclass;

  GB300P3MKernel() : Superclass() {}
  GB300P3MKernel(const GB300P3MKernel &o)
      : Superclass(o), m_DataDomain(o.m_DataDomain), m_Ratio(o.m_Ratio), m_Padding(o.m_Padding) {}
  GB300P3MKernel(const MatrixType &X, double h) : Superclass(X, h) {}
  GB300P3MKernel(const MatrixType &X, const MatrixType &W, double h) : Superclass(X, W, h) {}
  virtual GB300P3MKernel *Clone() const { return new GB300P3MKernel(*this); }
  virtual ~GB300P3MKernel() {}

  void SetDataDomain(MatrixType DD) { m_DataDomain = DD; }
  void SetWorkingSpacingRatio(const ScalarType d) { m_Ratio = d; }
  void SetPaddingFactor(const ScalarType d) { m_Padding = d; }

  virtual MatrixType Convolve(const MatrixType &X) {
    Call c(this, X);
    std::vector<double> out((size_t)X.rows() * c.dv);
    gb300_binding::check(gbk_p3m_convolve(gb300_binding::thread_context(), PointDim, c.dv, c.x.memptr(), X.rows(),
                                          c.y.memptr(), c.w.memptr(), c.ny, this->GetKernelWidth(), c.domain(),
                                          m_Ratio, m_Padding, out.data()));
    return rows(out, X.rows(), c.dv);
  }

  virtual std::vector<MatrixType> ConvolveGradient(const MatrixType &X) {
    Call c(this, X);
    std::vector<double> out((size_t)X.rows() * c.dv * PointDim);
    gb300_binding::check(gbk_p3m_convolve_gradient(gb300_binding::thread_context(), PointDim, c.dv, c.x.memptr(),
                                                   X.rows(), c.y.memptr(), c.w.memptr(), c.ny,
                                                   this->GetKernelWidth(), c.domain(), m_Ratio, m_Padding,
                                                   out.data()));
    std::vector<MatrixType> g;
    for (unsigned i = 0; i < X.rows(); ++i) {
      MatrixType Gi(c.dv, PointDim, 0.0);
      for (unsigned k = 0; k < c.dv; ++k)
        for (unsigned l = 0; l < PointDim; ++l) Gi(k, l) = out[((size_t)i * c.dv + k) * PointDim + l];
      g.push_back(Gi);
    }
    return g;
  }

  virtual MatrixType ConvolveGradient(const MatrixType &X, const MatrixType &alpha) {
    Call c(this, X);
    VectorType a = alpha.vectorise_row_wise();
    std::vector<double> out((size_t)X.rows() * PointDim);
    gb300_binding::check(gbk_p3m_convolve_gradient_alpha(gb300_binding::thread_context(), PointDim, c.dv,
                                                         c.x.memptr(), X.rows(), c.y.memptr(), c.w.memptr(), c.ny,
                                                         this->GetKernelWidth(), a.memptr(), c.domain(), m_Ratio,
                                                         m_Padding, out.data()));
    return rows(out, X.rows(), PointDim);
  }

  virtual VectorType ConvolveGradient(const MatrixType &X, unsigned int k, unsigned int dp) {
    Call c(this, X);
    std::vector<double> out(X.rows());
    gb300_binding::check(gbk_p3m_convolve_gradient_kdp(gb300_binding::thread_context(), PointDim, c.dv, X.rows(), c.ny,
                                                       (int)k, (int)dp, out.data()));
    return VectorType(out);
  }

  virtual MatrixType ConvolveGradient(const MatrixType &X, unsigned int dim) {
    Call c(this, X);
    std::vector<double> out((size_t)X.rows() * c.dv);
    gb300_binding::check(gbk_p3m_convolve_gradient_dim(gb300_binding::thread_context(), PointDim, c.dv,
                                                       c.x.memptr(), X.rows(), c.y.memptr(), c.w.memptr(), c.ny,
                                                       this->GetKernelWidth(), (int)dim, c.domain(), m_Ratio,
                                                       m_Padding, out.data()));
    return rows(out, X.rows(), c.dv);
  }

  virtual std::vector<std::vector<MatrixType> > ConvolveHessian(const MatrixType &X) {
    Call c(this, X);
    const unsigned D = PointDim;
    std::vector<double> out((size_t)X.rows() * c.dv * D * D);
    gb300_binding::check(gbk_p3m_convolve_hessian(gb300_binding::thread_context(), D, c.dv, c.x.memptr(), X.rows(),
                                                  c.y.memptr(), c.w.memptr(), c.ny, this->GetKernelWidth(),
                                                  c.domain(), m_Ratio, m_Padding, out.data()));
    std::vector<std::vector<MatrixType> > h;
    for (unsigned i = 0; i < X.rows(); ++i) {
      std::vector<MatrixType> Hi;
      for (unsigned k = 0; k < c.dv; ++k) {
        MatrixType H(D, D, 0.0);
        for (unsigned a = 0; a < D; ++a)
          for (unsigned b = 0; b < D; ++b) H(a, b) = out[(((size_t)i * c.dv + k) * D + a) * D + b];
        Hi.push_back(H);
      }
      h.push_back(Hi);
    }
    return h;
  }

  virtual VectorType ConvolveHessian(const MatrixType &X, unsigned int k, unsigned int dp, unsigned int dq) {
    Call c(this, X);
    std::vector<double> out(X.rows());
    gb300_binding::check(gbk_p3m_convolve_hessian_kdpdq(gb300_binding::thread_context(), PointDim, c.dv, X.rows(),
                                                        c.ny, (int)k, (int)dp, (int)dq, out.data()));
    return VectorType(out);
  }

  virtual MatrixType ConvolveHessian(const MatrixType &X, unsigned int row, unsigned int col) {
    Call c(this, X);
    std::vector<double> out((size_t)X.rows() * c.dv);
    gb300_binding::check(gbk_p3m_convolve_hessian_rowcol(gb300_binding::thread_context(), PointDim, c.dv,
                                                         c.x.memptr(), X.rows(), c.y.memptr(), c.w.memptr(), c.ny,
                                                         this->GetKernelWidth(), (int)row, (int)col, c.domain(),
                                                         m_Ratio, m_Padding, out.data()));
    return rows(out, X.rows(), c.dv);
  }

 private:
  MatrixType m_DataDomain;  // PointDim x 2 (empty: the bounding box of targets and sources)
  double m_Ratio = 0.2, m_Padding = 3.0;

  // row-major copies of the call's matrices and the domain as lo[PointDim], hi[PointDim]
  struct Call {
    VectorType x, y, w;
    std::vector<double> dom;
    unsigned ny, dv;
    Call(GB300P3MKernel *k, const MatrixType &X) {
      MatrixType &Y = k->GetSources();
      MatrixType &W = k->GetWeights();
      if (Y.rows() != W.rows()) throw std::runtime_error("Sources and weights count mismatch");
      x = X.vectorise_row_wise();
      y = Y.vectorise_row_wise();
      w = W.vectorise_row_wise();
      ny = Y.rows();
      dv = W.columns();
      if (k->m_DataDomain.rows() == PointDim && k->m_DataDomain.columns() == 2) {
        dom.resize(2 * PointDim);
        for (unsigned d = 0; d < PointDim; ++d) {
          dom[d] = k->m_DataDomain(d, 0);
          dom[PointDim + d] = k->m_DataDomain(d, 1);
        }
      }
    }
    const double *domain() const { return dom.empty() ? nullptr : dom.data(); }
  };

  static MatrixType rows(const std::vector<double> &v, unsigned n, unsigned cols) {
    MatrixType M(n, cols, 0.0);
    for (unsigned i = 0; i < n; ++i)
      for (unsigned j = 0; j < cols; ++j) M(i, j) = v[(size_t)i * cols + j];
    return M;
  }
};
