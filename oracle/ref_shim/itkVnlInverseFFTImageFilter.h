// Oracle-only stand-in for ITK 4's VnlInverseFFTImageFilter: the inverse DFT of a full-size complex
// image, real part divided by the number of pixels, as a real image with the input's origin,
// spacing and region (see itk_standin_dft.h).
#pragma once
#include "itkImage.h"
#include "itkImageRegionConstIteratorWithIndex.h"
#include "itk_standin_dft.h"
namespace itk {
template <class In> class VnlInverseFFTImageFilter {
 public:
  static constexpr unsigned D = In::ImageDimension;
  typedef Image<typename In::PixelType::value_type, D> OutputImageType;
  typedef SmartPointer<VnlInverseFFTImageFilter> Pointer;
  static Pointer New() { return Pointer(std::make_shared<VnlInverseFFTImageFilter>()); }
  void SetInput(const In *in) { m_Input = in; }
  void SetNumberOfThreads(int) {}
  void Update() {
    const auto region = m_Input->GetLargestPossibleRegion();
    std::vector<std::complex<double>> buf;
    buf.reserve(region.GetNumberOfPixels());
    for (ImageRegionConstIteratorWithIndex<In> it(m_Input, region); !it.IsAtEnd(); ++it) buf.push_back(it.Get());
    standin::dft<D>(buf, region.m_Size.v, +1);
    const double npix = (double)region.GetNumberOfPixels();
    m_Output = OutputImageType::New();
    m_Output->CopyInformation(m_Input);
    m_Output->Allocate();
    size_t i = 0;
    for (ImageRegionIteratorWithIndex<OutputImageType> it(m_Output, region); !it.IsAtEnd(); ++it)
      it.Set(buf[i++].real() / npix);
  }
  typename OutputImageType::Pointer GetOutput() const { return m_Output; }

 private:
  const In *m_Input = nullptr;
  typename OutputImageType::Pointer m_Output;
};
}  // namespace itk
