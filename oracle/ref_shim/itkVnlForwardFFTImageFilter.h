// Oracle-only stand-in for ITK 4's VnlForwardFFTImageFilter: the unnormalised forward DFT of a real
// image as a full-size complex image with the input's origin, spacing and region (see
// itk_standin_dft.h).
#pragma once
#include "itkImage.h"
#include "itkImageRegionConstIteratorWithIndex.h"
#include "itk_standin_dft.h"
namespace itk {
template <class In> class VnlForwardFFTImageFilter {
 public:
  static constexpr unsigned D = In::ImageDimension;
  typedef Image<std::complex<typename In::PixelType>, D> OutputImageType;
  typedef SmartPointer<VnlForwardFFTImageFilter> Pointer;
  static Pointer New() { return Pointer(std::make_shared<VnlForwardFFTImageFilter>()); }
  void SetInput(const In *in) { m_Input = in; }
  void SetNumberOfThreads(int) {}
  void Update() {
    const auto region = m_Input->GetLargestPossibleRegion();
    std::vector<std::complex<double>> buf;
    buf.reserve(region.GetNumberOfPixels());
    for (ImageRegionConstIteratorWithIndex<In> it(m_Input, region); !it.IsAtEnd(); ++it)
      buf.push_back(std::complex<double>(it.Get(), 0.0));
    standin::dft<D>(buf, region.m_Size.v, -1);
    m_Output = OutputImageType::New();
    m_Output->CopyInformation(m_Input);
    m_Output->Allocate();
    size_t i = 0;
    for (ImageRegionIteratorWithIndex<OutputImageType> it(m_Output, region); !it.IsAtEnd(); ++it) it.Set(buf[i++]);
  }
  typename OutputImageType::Pointer GetOutput() const { return m_Output; }

 private:
  const In *m_Input = nullptr;
  typename OutputImageType::Pointer m_Output;
};
}  // namespace itk
