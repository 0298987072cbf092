// Oracle-only stand-in (see itkImage.h): compiles, throws if used.
#pragma once
#include "itkImage.h"
namespace itk {
template <class ImageT> class ImageRegionConstIteratorWithIndex {
 public:
  template <class P, class R> ImageRegionConstIteratorWithIndex(const P &, const R &) {
    throw std::runtime_error("ITK stand-in: not available in the oracle");
  }
  bool IsAtEnd() const { return true; }
  Index<ImageT::ImageDimension> GetIndex() const { return Index<ImageT::ImageDimension>(); }
  ImageRegionConstIteratorWithIndex &operator++() { return *this; }
};
}
