// Oracle-only stand-in (see itkImage.h): visits a region of an image, first index fastest; throws
// when the region is not inside the image.
#pragma once
#include "itkImage.h"
namespace itk {
template <class ImageT> class ImageRegionConstIteratorWithIndex {
 public:
  static constexpr unsigned D = ImageT::ImageDimension;
  template <class P>
  ImageRegionConstIteratorWithIndex(const P &image, const ImageRegion<D> &region) : m_Region(region) {
    if (!image->GetLargestPossibleRegion().IsInside(region))
      throw std::runtime_error("ITK stand-in: region is outside of the image");
    m_Index = region.m_Index;
    m_End = false;
    for (unsigned i = 0; i < D; ++i) m_End = m_End || region.m_Size[i] == 0;
  }
  bool IsAtEnd() const { return m_End; }
  Index<D> GetIndex() const { return m_Index; }
  ImageRegionConstIteratorWithIndex &operator++() {
    for (unsigned i = 0; i < D; ++i) {
      if (++m_Index[i] < m_Region.m_Index[i] + (long)m_Region.m_Size[i]) return *this;
      m_Index[i] = m_Region.m_Index[i];
    }
    m_End = true;
    return *this;
  }

 private:
  ImageRegion<D> m_Region;
  Index<D> m_Index;
  bool m_End;
};
}  // namespace itk
