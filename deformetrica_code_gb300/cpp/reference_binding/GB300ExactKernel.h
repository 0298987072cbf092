// GB300ExactKernel.h -- the kernel type a Deformetrica build adds to use the GB300 library.
//
// Drop-in beside src/support/kernels/CUDAExactKernel.h: it derives from ExactKernel because the
// factory's base type is ExactKernel (KernelFactory.h:44), and overrides every convolution method
// of AbstractKernel (AbstractKernel.h:120-165), the image-grid ones included, so no call falls back
// to the CPU loops. Each method
// builds the row-major buffers the legacy CUDA path builds (vectorise_row_wise,
// CUDAExactKernel.cxx:46-48) and makes one call into the C ABI of include/gbk.h; failures throw
// std::runtime_error with the library's message, as the reference does for shape errors. One
// library context per host thread (kernel objects are created per subject thread,
// AbstractAtlas.cxx:218), lazily created on first use.
//
// Selecting it takes an enum value GB300Exact in KernelType.h:20-28 and one case in each
// KernelFactory::CreateKernelObject overload (KernelFactory.cxx:100-117, 128-144, 155-171), plus the
// kernel-type strings of the launchers and of DeformableObjectReader.cxx:473-485.
#pragma once

#include <cstdlib>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ExactKernel.h"
#include "gbk.h"

namespace gb300_binding {

// The library context of the calling thread, created on first use on the GPU named by the
// environment variable GBK_DEVICE (default 0) in the precision named by GBK_MODE ("f64" for the FP64
// mode, anything else the default compensated FP32).
inline gbk_ctx *thread_context() {
  struct Holder {
    gbk_ctx *c = nullptr;
    ~Holder() {
      if (c) gbk_destroy(c);
    }
  };
  static thread_local Holder h;
  if (!h.c) {
    const char *dev = std::getenv("GBK_DEVICE");
    const char *mode = std::getenv("GBK_MODE");
    if (gbk_create(dev ? std::atoi(dev) : 0, &h.c) != GBK_OK)
      throw std::runtime_error(std::string("gbk_create: ") + gbk_last_error(nullptr));
    if (mode && std::string(mode) == "f64" && gbk_set_mode(h.c, GBK_MODE_F64) != GBK_OK)
      throw std::runtime_error(gbk_last_error(h.c));
  }
  return h.c;
}

inline void check(int rc) {
  if (rc != GBK_OK) throw std::runtime_error(gbk_last_error(thread_context()));
}

}  // namespace gb300_binding

template <class ScalarType, unsigned int PointDim>
class GB300ExactKernel : public ExactKernel<ScalarType, PointDim> {
 public:
  typedef ExactKernel<ScalarType, PointDim> Superclass;

  GB300ExactKernel() : Superclass() {}
  // a copy uploads its own device copies on first use
  GB300ExactKernel(const GB300ExactKernel &o) : Superclass(o) {}
  GB300ExactKernel(const MatrixType &X, double h) : Superclass(X, h) {}
  GB300ExactKernel(const MatrixType &X, const MatrixType &W, double h) : Superclass(X, W, h) {}
  virtual GB300ExactKernel *Clone() const { return new GB300ExactKernel(*this); }
  virtual ~GB300ExactKernel() {
    gbk_buffer_destroy(m_DeviceSources);
    gbk_buffer_destroy(m_DeviceWeights);
  }

  // Uploads of the sources so far (for tests: SetSources, SetWeights or SetKernelWidth mark the object
  // modified and the next call uploads again; calls in between reuse the device copies).
  long long SourceUploads() const { return m_DeviceSources ? gbk_buffer_uploads(m_DeviceSources) : 0; }

  virtual MatrixType Convolve(const MatrixType &X) {
    Buffers b(this, X);
    std::vector<double> out((size_t)X.rows() * b.dv);
    gb300_binding::check(gbk_convolve(gb300_binding::thread_context(), PointDim, b.dv, b.x.memptr(), X.rows(),
                                      b.y, b.w, b.ny, this->GetKernelWidth(), out.data()));
    return from_rows(out, X.rows(), b.dv);
  }

  virtual std::vector<MatrixType> ConvolveGradient(const MatrixType &X) {
    Buffers b(this, X);
    std::vector<double> out((size_t)X.rows() * b.dv * PointDim);
    gb300_binding::check(gbk_convolve_gradient(gb300_binding::thread_context(), PointDim, b.dv, b.x.memptr(),
                                               X.rows(), b.y, b.w, b.ny,
                                               this->GetKernelWidth(), out.data()));
    std::vector<MatrixType> g;
    for (unsigned i = 0; i < X.rows(); ++i) {
      MatrixType Gi(b.dv, PointDim, 0.0);
      for (unsigned k = 0; k < b.dv; ++k)
        for (unsigned l = 0; l < PointDim; ++l) Gi(k, l) = out[((size_t)i * b.dv + k) * PointDim + l];
      g.push_back(Gi);
    }
    return g;
  }

  virtual MatrixType ConvolveGradient(const MatrixType &X, const MatrixType &alpha) {
    Buffers b(this, X);
    VectorType a = alpha.vectorise_row_wise();
    std::vector<double> out((size_t)X.rows() * PointDim);
    gb300_binding::check(gbk_convolve_gradient_alpha(gb300_binding::thread_context(), PointDim, b.dv,
                                                     b.x.memptr(), X.rows(), b.y, b.w, b.ny,
                                                     this->GetKernelWidth(), a.memptr(), out.data()));
    return from_rows(out, X.rows(), PointDim);
  }

  virtual VectorType ConvolveGradient(const MatrixType &X, unsigned int k, unsigned int dp) {
    Buffers b(this, X);
    std::vector<double> out(b.ny);
    gb300_binding::check(gbk_convolve_gradient_kdp(gb300_binding::thread_context(), PointDim, b.dv,
                                                   b.x.memptr(), X.rows(), b.y, b.w, b.ny,
                                                   this->GetKernelWidth(), (int)k, (int)dp, out.data()));
    return VectorType(out);
  }

  virtual MatrixType ConvolveGradient(const MatrixType &X, unsigned int dim) {
    Buffers b(this, X);
    std::vector<double> out((size_t)X.rows() * b.dv);
    gb300_binding::check(gbk_convolve_gradient_dim(gb300_binding::thread_context(), PointDim, b.dv,
                                                   b.x.memptr(), X.rows(), b.y, b.w, b.ny,
                                                   this->GetKernelWidth(), (int)dim, out.data()));
    return from_rows(out, X.rows(), b.dv);
  }

  virtual std::vector<std::vector<MatrixType> > ConvolveHessian(const MatrixType &X) {
    Buffers b(this, X);
    const unsigned D = PointDim;
    std::vector<double> out((size_t)X.rows() * b.dv * D * D);
    gb300_binding::check(gbk_convolve_hessian(gb300_binding::thread_context(), D, b.dv, b.x.memptr(), X.rows(),
                                              b.y, b.w, b.ny, this->GetKernelWidth(),
                                              out.data()));
    std::vector<std::vector<MatrixType> > h;
    for (unsigned i = 0; i < X.rows(); ++i) {
      std::vector<MatrixType> Hi;
      for (unsigned k = 0; k < b.dv; ++k) {
        MatrixType H(D, D, 0.0);
        for (unsigned a = 0; a < D; ++a)
          for (unsigned c = 0; c < D; ++c) H(a, c) = out[(((size_t)i * b.dv + k) * D + a) * D + c];
        Hi.push_back(H);
      }
      h.push_back(Hi);
    }
    return h;
  }

  virtual VectorType ConvolveHessian(const MatrixType &X, unsigned int k, unsigned int dp, unsigned int dq) {
    Buffers b(this, X);
    std::vector<double> out(X.rows());
    gb300_binding::check(gbk_convolve_hessian_kdpdq(gb300_binding::thread_context(), PointDim, b.dv,
                                                    b.x.memptr(), X.rows(), b.y, b.w, b.ny,
                                                    this->GetKernelWidth(), (int)k, (int)dp, (int)dq, out.data()));
    return VectorType(out);
  }

  virtual MatrixType ConvolveHessian(const MatrixType &X, unsigned int row, unsigned int col) {
    Buffers b(this, X);
    std::vector<double> out((size_t)X.rows() * b.dv);
    gb300_binding::check(gbk_convolve_hessian_rowcol(gb300_binding::thread_context(), PointDim, b.dv,
                                                     b.x.memptr(), X.rows(), b.y, b.w, b.ny,
                                                     this->GetKernelWidth(), (int)row, (int)col, out.data()));
    return from_rows(out, X.rows(), b.dv);
  }

  virtual MatrixType ConvolveSpecialHessian(const MatrixType &xi) {
    Buffers b(this, this->GetSources());
    if (xi.rows() != b.ny) throw std::runtime_error("Y and Xi count mismatch");
    VectorType x = xi.vectorise_row_wise();
    std::vector<double> out((size_t)b.ny * PointDim);
    gb300_binding::check(gbk_convolve_special_hessian(gb300_binding::thread_context(), PointDim, b.y,
                                                      b.w, b.ny, this->GetKernelWidth(), x.memptr(),
                                                      out.data()));
    return from_rows(out, b.ny, PointDim);
  }

  // ExactKernel::ConvolveImageFast (ExactKernel.cxx:76-129) on the device: the image's origin,
  // spacing and size go to the C ABI; images with a non-identity direction are refused (the
  // library's pixel geometry is origin + spacing x index).
  virtual MatrixType ConvolveImageFast(const MatrixType &X, const typename Superclass::ImageTypePointer image) {
    Buffers b(this, X);
    if (b.dv != PointDim) throw std::runtime_error("ConvolveImageFast needs weights with PointDim columns");
    const Geometry g(image);
    std::vector<double> out((size_t)X.rows() * PointDim);
    gb300_binding::check(gbk_convolve_image_fast(gb300_binding::thread_context(), PointDim, b.x.memptr(), X.rows(),
                                                 b.y, b.w, b.ny, this->GetKernelWidth(), g.o, g.s, g.n,
                                                 out.data()));
    return from_rows(out, X.rows(), PointDim);
  }

  // ExactKernel::ConvolveGradientImageFast(X, image) (ExactKernel.cxx:207-257): one dv x PointDim
  // matrix per pixel, over the same windows.
  virtual std::vector<MatrixType> ConvolveGradientImageFast(const MatrixType &X,
                                                            const typename Superclass::ImageTypePointer image) {
    Buffers b(this, X);
    const Geometry g(image);
    std::vector<double> out((size_t)X.rows() * b.dv * PointDim);
    gb300_binding::check(gbk_convolve_gradient_image_fast(gb300_binding::thread_context(), PointDim, b.dv,
                                                          b.x.memptr(), X.rows(), b.y, b.w, b.ny,
                                                          this->GetKernelWidth(), g.o, g.s, g.n, out.data()));
    std::vector<MatrixType> grad;
    for (unsigned i = 0; i < X.rows(); ++i) {
      MatrixType Gi(b.dv, PointDim, 0.0);
      for (unsigned k = 0; k < b.dv; ++k)
        for (unsigned l = 0; l < PointDim; ++l) Gi(k, l) = out[((size_t)i * b.dv + k) * PointDim + l];
      grad.push_back(Gi);
    }
    return grad;
  }

  // ExactKernel::ConvolveGradientImageFast(X, alpha, image) (ExactKernel.cxx:277-290): G_p^T alpha_p.
  virtual MatrixType ConvolveGradientImageFast(const MatrixType &X, const MatrixType &alpha,
                                               const typename Superclass::ImageTypePointer image) {
    Buffers b(this, X);
    if (alpha.rows() != X.rows() || alpha.columns() != b.dv) throw std::runtime_error("alpha size mismatch");
    const Geometry g(image);
    VectorType a = alpha.vectorise_row_wise();
    std::vector<double> out((size_t)X.rows() * PointDim);
    gb300_binding::check(gbk_convolve_gradient_image_fast_alpha(
        gb300_binding::thread_context(), PointDim, b.dv, b.x.memptr(), X.rows(), b.y, b.w, b.ny,
        this->GetKernelWidth(), a.memptr(), g.o, g.s, g.n, out.data()));
    return from_rows(out, X.rows(), PointDim);
  }

 private:
  // An ITK image's origin, spacing and size for the C ABI; identity direction only.
  struct Geometry {
    double o[PointDim], s[PointDim];
    long n[PointDim];
    explicit Geometry(const typename Superclass::ImageTypePointer &image) {
      const auto origin = image->GetOrigin();
      const auto spacing = image->GetSpacing();
      const auto direction = image->GetDirection();
      const auto size = image->GetLargestPossibleRegion().GetSize();
      for (unsigned i = 0; i < PointDim; ++i) {
        o[i] = origin[i];
        s[i] = spacing[i];
        n[i] = (long)size[i];
        for (unsigned j = 0; j < PointDim; ++j)
          if (direction[i][j] != (i == j ? 1.0 : 0.0))
            throw std::runtime_error("GB300ExactKernel: image with a non-identity direction");
      }
    }
  };

  // The call's targets as a row-major host array and the device copies of the sources and weights,
  // uploaded only when the object is modified (m_Modified, AbstractKernel.h:172-185: SetSources,
  // SetWeights and SetKernelWidth set it; as for the reference's P3MKernel, matrices changed in
  // place through GetSources() / GetWeights() are not seen until one of those is called).
  struct Buffers {
    VectorType x;
    const double *y = nullptr, *w = nullptr;
    unsigned ny, dv;
    Buffers(GB300ExactKernel *k, const MatrixType &X) {
      MatrixType &Y = k->GetSources();
      MatrixType &W = k->GetWeights();
      if (Y.rows() != W.rows()) throw std::runtime_error("Sources and weights count mismatch");
      x = X.vectorise_row_wise();
      ny = Y.rows();
      dv = W.columns();
      gbk_ctx *c = gb300_binding::thread_context();
      if (!k->m_DeviceSources) gb300_binding::check(gbk_buffer_create(c, &k->m_DeviceSources));
      if (!k->m_DeviceWeights) gb300_binding::check(gbk_buffer_create(c, &k->m_DeviceWeights));
      if (k->IsModified() || gbk_buffer_uploads(k->m_DeviceSources) == 0) {
        VectorType yv = Y.vectorise_row_wise(), wv = W.vectorise_row_wise();
        gb300_binding::check(gbk_buffer_upload(c, k->m_DeviceSources, yv.memptr(), (size_t)ny * PointDim));
        gb300_binding::check(gbk_buffer_upload(c, k->m_DeviceWeights, wv.memptr(), (size_t)ny * dv));
        k->UnsetModified();
      }
      y = gbk_buffer_data(k->m_DeviceSources);
      w = gbk_buffer_data(k->m_DeviceWeights);
    }
  };

  gbk_buffer *m_DeviceSources = nullptr;
  gbk_buffer *m_DeviceWeights = nullptr;

  static MatrixType from_rows(const std::vector<double> &v, unsigned rows, unsigned cols) {
    MatrixType M(rows, cols, 0.0);
    for (unsigned i = 0; i < rows; ++i)
      for (unsigned j = 0; j < cols; ++j) M(i, j) = v[(size_t)i * cols + j];
    return M;
  }
};
