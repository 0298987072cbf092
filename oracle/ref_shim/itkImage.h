// Oracle-only stand-ins for the ITK image types the reference's kernel code names (test
// infrastructure; ITK itself is not available here). They implement, for images with an identity
// direction, the documented behaviour that ExactKernel::ConvolveImageFast and
// ConvolveGradientImageFast (src/support/kernels/ExactKernel.cxx:76-129, 207-290) rely on:
//  * Size::Fill stores one value on every axis (the caller's double converts to the unsigned size
//    type, i.e. truncates, as with ITK's SizeValueType);
//  * Image::TransformPhysicalPointToIndex maps a physical point to the index
//    RoundHalfIntegerUp((point - origin) / spacing) on each axis (ITK multiplies by the inverse of
//    diag(spacing), computed numerically, so exact half-integer ties may round differently there);
//  * ImageRegion::Crop clips a region to another one, leaves it unchanged and returns false when
//    they do not overlap;
//  * the region iterator (itkImageRegionConstIteratorWithIndex.h) visits the region's indices with
//    the first index fastest, and throws when the region is not inside the image (ITK's iterators
//    throw for a region outside the buffered region).
// Images are made with the driver-only constructor Image(origin, spacing, size).
#pragma once
#include <cmath>
#include <memory>
#include <stdexcept>
namespace itk {
template <unsigned D> struct Size {
  unsigned long v[D];
  void Fill(unsigned long x) { for (unsigned i = 0; i < D; ++i) v[i] = x; }
  unsigned long &operator[](unsigned i) { return v[i]; }
  const unsigned long &operator[](unsigned i) const { return v[i]; }
};
template <unsigned D> struct Index {
  long v[D];
  long &operator[](unsigned i) { return v[i]; }
  const long &operator[](unsigned i) const { return v[i]; }
};
template <class T, unsigned D> struct Point {
  T v[D];
  T &operator[](unsigned i) { return v[i]; }
  const T &operator[](unsigned i) const { return v[i]; }
};
template <unsigned D> struct ImageRegion {
  Index<D> m_Index{};
  Size<D> m_Size{};
  ImageRegion() {}
  ImageRegion(const Index<D> &index, const Size<D> &size) : m_Index(index), m_Size(size) {}
  Size<D> GetSize() const { return m_Size; }
  Index<D> GetIndex() const { return m_Index; }
  bool Crop(const ImageRegion &r) {
    for (unsigned i = 0; i < D; ++i)
      if (m_Index[i] >= r.m_Index[i] + (long)r.m_Size[i] || m_Index[i] + (long)m_Size[i] <= r.m_Index[i]) return false;
    for (unsigned i = 0; i < D; ++i) {
      if (m_Index[i] < r.m_Index[i]) {
        const long crop = r.m_Index[i] - m_Index[i];
        m_Index[i] += crop;
        m_Size[i] -= (unsigned long)crop;
      }
      const long end = m_Index[i] + (long)m_Size[i], rend = r.m_Index[i] + (long)r.m_Size[i];
      if (end > rend) m_Size[i] -= (unsigned long)(end - rend);
    }
    return true;
  }
  bool IsInside(const ImageRegion &r) const {  // r inside *this
    for (unsigned i = 0; i < D; ++i)
      if (r.m_Index[i] < m_Index[i] || r.m_Index[i] + (long)r.m_Size[i] > m_Index[i] + (long)m_Size[i]) return false;
    return true;
  }
};
template <class T, unsigned D> class Image {
 public:
  typedef std::shared_ptr<Image> Pointer;
  typedef T PixelType;
  static constexpr unsigned ImageDimension = D;
  struct Vec {
    double v[D];
    double operator[](unsigned i) const { return v[i]; }
  };
  struct Mat {
    double v[D][D];
    const double *operator[](unsigned i) const { return v[i]; }
  };
  Image() {
    for (unsigned i = 0; i < D; ++i) {
      m_Origin.v[i] = 0.0;
      m_Spacing.v[i] = 1.0;
      m_Region.m_Index[i] = 0;
      m_Region.m_Size[i] = 1;
    }
  }
  Image(const double *origin, const double *spacing, const long *size) : Image() {
    for (unsigned i = 0; i < D; ++i) {
      m_Origin.v[i] = origin[i];
      m_Spacing.v[i] = spacing[i];
      m_Region.m_Size[i] = (unsigned long)size[i];
    }
  }
  ImageRegion<D> GetLargestPossibleRegion() const { return m_Region; }
  Vec GetOrigin() const { return m_Origin; }
  Vec GetSpacing() const { return m_Spacing; }
  Mat GetDirection() const {
    Mat m;
    for (unsigned i = 0; i < D; ++i)
      for (unsigned j = 0; j < D; ++j) m.v[i][j] = i == j ? 1.0 : 0.0;
    return m;
  }
  template <class P, class I> bool TransformPhysicalPointToIndex(const P &point, I &index) const {
    bool inside = true;
    for (unsigned i = 0; i < D; ++i) {
      index[i] = (long)std::floor((point[i] - m_Origin.v[i]) / m_Spacing.v[i] + 0.5);
      inside = inside && index[i] >= 0 && index[i] < (long)m_Region.m_Size[i];
    }
    return inside;
  }

 private:
  Vec m_Origin, m_Spacing;
  ImageRegion<D> m_Region;
};
}  // namespace itk
