// Oracle-only stand-ins for the ITK image types the reference's kernel code names (test
// infrastructure; ITK itself is not available here). They implement, for images with an identity
// direction, the documented behaviour that ExactKernel::ConvolveImageFast and
// ConvolveGradientImageFast (src/support/kernels/ExactKernel.cxx:76-129, 207-290) and P3MKernel
// (src/support/kernels/P3MKernel.cxx) rely on:
//  * Size::Fill stores one value on every axis (the caller's double converts to the unsigned size
//    type, i.e. truncates, as with ITK's SizeValueType);
//  * Image::TransformPhysicalPointToIndex maps a physical point to the index
//    RoundHalfIntegerUp((point - origin) / spacing) on each axis (ITK multiplies by the inverse of
//    diag(spacing), computed numerically, so exact half-integer ties may round differently there);
//    TransformIndexToPhysicalPoint maps an index to origin + spacing * index;
//  * ImageRegion::Crop clips a region to another one, leaves it unchanged and returns false when
//    they do not overlap;
//  * pixel buffers (Allocate, FillBuffer, GetPixel, SetPixel) are stored with the first index
//    fastest; CopyInformation copies the origin, spacing and largest possible region;
//  * the region iterators (itkImageRegion*IteratorWithIndex.h) visit the region's indices with the
//    first index fastest, and throw when the region is not inside the image (ITK's iterators
//    throw for a region outside the buffered region).
// Pointers are shared pointers that also convert to raw pointers, as ITK's SmartPointer does.
// Images without a buffer can be made with the driver-only constructor Image(origin, spacing, size).
#pragma once
#include <cmath>
#include <complex>
#include <cstddef>
#include <memory>
#include <ostream>
#include <stdexcept>
#include <vector>

namespace vnl_math {
constexpr double pi = 3.14159265358979323846;
}

namespace itk {
template <class T> class SmartPointer : public std::shared_ptr<T> {
 public:
  SmartPointer() = default;
  SmartPointer(std::nullptr_t) {}
  SmartPointer(std::shared_ptr<T> p) : std::shared_ptr<T>(std::move(p)) {}
  operator T *() const { return this->get(); }
};

template <unsigned D> struct Size {
  unsigned long v[D];
  void Fill(unsigned long x) { for (unsigned i = 0; i < D; ++i) v[i] = x; }
  unsigned long &operator[](unsigned i) { return v[i]; }
  const unsigned long &operator[](unsigned i) const { return v[i]; }
};
template <unsigned D> struct Index {
  long v[D];
  void Fill(long x) { for (unsigned i = 0; i < D; ++i) v[i] = x; }
  long &operator[](unsigned i) { return v[i]; }
  const long &operator[](unsigned i) const { return v[i]; }
};
template <class T, unsigned D> struct Point {
  T v[D];
  void Fill(T x) { for (unsigned i = 0; i < D; ++i) v[i] = x; }
  T &operator[](unsigned i) { return v[i]; }
  const T &operator[](unsigned i) const { return v[i]; }
};
template <unsigned D> std::ostream &operator<<(std::ostream &os, const Size<D> &s) {
  os << "[";
  for (unsigned i = 0; i < D; ++i) os << (i ? ", " : "") << s[i];
  return os << "]";
}
template <class T, unsigned D> std::ostream &operator<<(std::ostream &os, const Point<T, D> &p) {
  os << "[";
  for (unsigned i = 0; i < D; ++i) os << (i ? ", " : "") << p[i];
  return os << "]";
}

template <unsigned D> struct ImageRegion {
  Index<D> m_Index{};
  Size<D> m_Size{};
  ImageRegion() {}
  ImageRegion(const Index<D> &index, const Size<D> &size) : m_Index(index), m_Size(size) {}
  Size<D> GetSize() const { return m_Size; }
  Index<D> GetIndex() const { return m_Index; }
  void SetSize(const Size<D> &s) { m_Size = s; }
  void SetIndex(const Index<D> &i) { m_Index = i; }
  unsigned long GetNumberOfPixels() const {
    unsigned long n = 1;
    for (unsigned i = 0; i < D; ++i) n *= m_Size[i];
    return n;
  }
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
  bool IsInside(const Index<D> &ind) const {
    for (unsigned i = 0; i < D; ++i)
      if (ind[i] < m_Index[i] || ind[i] >= m_Index[i] + (long)m_Size[i]) return false;
    return true;
  }
};

template <class T, unsigned D> class Image {
 public:
  typedef SmartPointer<Image> Pointer;
  typedef T PixelType;
  typedef Index<D> IndexType;
  typedef Size<D> SizeType;
  typedef ImageRegion<D> RegionType;
  typedef Point<double, D> PointType;
  typedef Point<double, D> SpacingType;  // ITK: Vector<double, D>
  static constexpr unsigned ImageDimension = D;
  struct Mat {
    double v[D][D];
    const double *operator[](unsigned i) const { return v[i]; }
  };
  static Pointer New() { return Pointer(std::make_shared<Image>()); }
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
  RegionType GetLargestPossibleRegion() const { return m_Region; }
  PointType GetOrigin() const { return m_Origin; }
  SpacingType GetSpacing() const { return m_Spacing; }
  Mat GetDirection() const {
    Mat m;
    for (unsigned i = 0; i < D; ++i)
      for (unsigned j = 0; j < D; ++j) m.v[i][j] = i == j ? 1.0 : 0.0;
    return m;
  }
  void SetRegions(const RegionType &r) { m_Region = r; }
  void SetOrigin(const PointType &o) { m_Origin = o; }
  void SetSpacing(const SpacingType &s) { m_Spacing = s; }
  template <class P> void CopyInformation(const P &other) {  // a raw or smart pointer to an image
    m_Origin = other->GetOrigin();
    m_Spacing = other->GetSpacing();
    m_Region = other->GetLargestPossibleRegion();
  }
  void Allocate() { m_Buffer.assign(m_Region.GetNumberOfPixels(), T()); }
  void FillBuffer(const T &v) { std::fill(m_Buffer.begin(), m_Buffer.end(), v); }
  void ReleaseDataFlagOff() {}
  T GetPixel(const IndexType &ind) const { return m_Buffer.at(Offset(ind)); }
  void SetPixel(const IndexType &ind, const T &v) { m_Buffer.at(Offset(ind)) = v; }
  T &Pixel(const IndexType &ind) { return m_Buffer.at(Offset(ind)); }
  // Offset of an index in the buffer, first index fastest; throws outside the region.
  size_t Offset(const IndexType &ind) const {
    if (!m_Region.IsInside(ind)) throw std::out_of_range("ITK stand-in: pixel index outside the image");
    size_t off = 0, stride = 1;
    for (unsigned i = 0; i < D; ++i) {
      off += (size_t)(ind[i] - m_Region.m_Index[i]) * stride;
      stride *= m_Region.m_Size[i];
    }
    return off;
  }
  template <class P, class I> bool TransformPhysicalPointToIndex(const P &point, I &index) const {
    bool inside = true;
    for (unsigned i = 0; i < D; ++i) {
      index[i] = (long)std::floor((point[i] - m_Origin.v[i]) / m_Spacing.v[i] + 0.5);
      inside = inside && index[i] >= 0 && index[i] < (long)m_Region.m_Size[i];
    }
    return inside;
  }
  template <class I, class P> void TransformIndexToPhysicalPoint(const I &index, P &point) const {
    for (unsigned i = 0; i < D; ++i) point[i] = m_Origin.v[i] + m_Spacing.v[i] * (double)index[i];
  }

 private:
  PointType m_Origin, m_Spacing;
  RegionType m_Region;
  std::vector<T> m_Buffer;
};
}  // namespace itk
