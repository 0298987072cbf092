// Oracle-only stand-in (see itkImage.h): visits a region of an image, first index fastest; throws
// when the region is not inside the image. ImageRegionIteratorWithIndex (same order) also sets
// pixels.
#pragma once
#include "itkImage.h"
namespace itk {
template <class ImageT> class ImageRegionConstIteratorWithIndex {
 public:
  static constexpr unsigned D = ImageT::ImageDimension;
  template <class P>
  ImageRegionConstIteratorWithIndex(const P &image, const ImageRegion<D> &region)
      : m_Image(&*image), m_Region(region) {
    if (!image->GetLargestPossibleRegion().IsInside(region))
      throw std::runtime_error("ITK stand-in: region is outside of the image");
    GoToBegin();
  }
  void GoToBegin() {
    m_Index = m_Region.m_Index;
    m_End = false;
    for (unsigned i = 0; i < D; ++i) m_End = m_End || m_Region.m_Size[i] == 0;
  }
  bool IsAtEnd() const { return m_End; }
  Index<D> GetIndex() const { return m_Index; }
  typename ImageT::PixelType Get() const { return m_Image->GetPixel(m_Index); }
  ImageRegionConstIteratorWithIndex &operator++() {
    for (unsigned i = 0; i < D; ++i) {
      if (++m_Index[i] < m_Region.m_Index[i] + (long)m_Region.m_Size[i]) return *this;
      m_Index[i] = m_Region.m_Index[i];
    }
    m_End = true;
    return *this;
  }

 protected:
  const ImageT *m_Image;
  ImageRegion<D> m_Region;
  Index<D> m_Index;
  bool m_End;
};

template <class ImageT> class ImageRegionIteratorWithIndex : public ImageRegionConstIteratorWithIndex<ImageT> {
 public:
  template <class P>
  ImageRegionIteratorWithIndex(const P &image, const ImageRegion<ImageT::ImageDimension> &region)
      : ImageRegionConstIteratorWithIndex<ImageT>(image, region), m_Mutable(&*image) {}
  void Set(const typename ImageT::PixelType &v) const { m_Mutable->SetPixel(this->m_Index, v); }
  ImageRegionIteratorWithIndex &operator++() {
    ImageRegionConstIteratorWithIndex<ImageT>::operator++();
    return *this;
  }

 private:
  ImageT *m_Mutable;
};
}  // namespace itk
