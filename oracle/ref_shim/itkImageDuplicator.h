// Oracle-only stand-in for ITK's ImageDuplicator: a deep copy of an image (information and pixels).
#pragma once
#include "itkImage.h"
namespace itk {
template <class ImageT> class ImageDuplicator {
 public:
  typedef SmartPointer<ImageDuplicator> Pointer;
  static Pointer New() { return Pointer(std::make_shared<ImageDuplicator>()); }
  void SetInputImage(const ImageT *in) { m_Input = in; }
  void Update() { m_Output = typename ImageT::Pointer(std::make_shared<ImageT>(*m_Input)); }
  typename ImageT::Pointer GetOutput() const { return m_Output; }

 private:
  const ImageT *m_Input = nullptr;
  typename ImageT::Pointer m_Output;
};
}  // namespace itk
