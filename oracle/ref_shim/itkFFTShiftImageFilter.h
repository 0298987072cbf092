// Oracle-only stand-in for ITK's FFTShiftImageFilter: a cyclic shift by half the size on every
// axis, out[k] = in[(k + n/2) mod n]. For even sizes (the only ones P3MKernel's power-of-two grids
// have, besides 1) the forward and the inverse shift are this same map; odd sizes above 1 throw.
#pragma once
#include <stdexcept>
#include "itkImage.h"
#include "itkImageRegionConstIteratorWithIndex.h"
namespace itk {
template <class In, class Out> class FFTShiftImageFilter {
 public:
  static constexpr unsigned D = In::ImageDimension;
  typedef SmartPointer<FFTShiftImageFilter> Pointer;
  static Pointer New() { return Pointer(std::make_shared<FFTShiftImageFilter>()); }
  void SetInput(const In *in) { m_Input = in; }
  void SetInverse(bool) {}
  void SetNumberOfThreads(int) {}
  void Update() {
    const auto region = m_Input->GetLargestPossibleRegion();
    for (unsigned i = 0; i < D; ++i)
      if (region.m_Size[i] > 1 && region.m_Size[i] % 2)
        throw std::runtime_error("ITK stand-in: FFT shift of an odd size");
    m_Output = Out::New();
    m_Output->CopyInformation(m_Input);
    m_Output->Allocate();
    for (ImageRegionIteratorWithIndex<Out> it(m_Output, region); !it.IsAtEnd(); ++it) {
      Index<D> src = it.GetIndex();
      for (unsigned i = 0; i < D; ++i) {
        const long n = (long)region.m_Size[i], lo = region.m_Index[i];
        src[i] = lo + ((src[i] - lo) + n / 2) % n;
      }
      it.Set(m_Input->GetPixel(src));
    }
  }
  typename Out::Pointer GetOutput() const { return m_Output; }

 private:
  const In *m_Input = nullptr;
  typename Out::Pointer m_Output;
};
}  // namespace itk
