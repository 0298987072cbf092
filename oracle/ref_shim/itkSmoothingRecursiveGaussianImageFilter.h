// Oracle-only stand-in: P3MKernel::ApplyKernelFFT names this filter on its path without a kernel
// image, which no P3MKernel method takes (they always pass the kernel spectra). Running it throws.
#pragma once
#include <stdexcept>
#include "itkImage.h"
namespace itk {
template <class In, class Out> class SmoothingRecursiveGaussianImageFilter {
 public:
  typedef SmartPointer<SmoothingRecursiveGaussianImageFilter> Pointer;
  static Pointer New() { return Pointer(std::make_shared<SmoothingRecursiveGaussianImageFilter>()); }
  void SetInput(const In *) {}
  void SetSigma(double) {}
  void SetNormalizeAcrossScale(bool) {}
  void Update() { throw std::runtime_error("ITK stand-in: recursive Gaussian smoothing is not available"); }
  typename Out::Pointer GetOutput() const { return typename Out::Pointer(); }
};
}  // namespace itk
