// Oracle-only stand-ins for the few ITK image types named by the kernel headers.
// The image-grid convolution (ConvolveImageFast) is outside the oracle's scope: these types
// exist so the explicit template instantiations compile, and every method throws if reached.
#pragma once
#include <stdexcept>
#include <memory>
namespace itk {
template <unsigned D> struct Size {
  unsigned long v[D];
  void Fill(double x) { for (unsigned i = 0; i < D; ++i) v[i] = (unsigned long)x; }
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
  ImageRegion() {}
  ImageRegion(const Index<D> &, const Size<D> &) {}
  Size<D> GetSize() const { throw std::runtime_error("ITK stand-in: not available in the oracle"); }
  bool Crop(const ImageRegion &) { throw std::runtime_error("ITK stand-in: not available in the oracle"); }
};
template <class T, unsigned D> class Image {
 public:
  typedef std::shared_ptr<Image> Pointer;
  typedef T PixelType;
  static constexpr unsigned ImageDimension = D;
  ImageRegion<D> GetLargestPossibleRegion() const { throw std::runtime_error("ITK stand-in: not available in the oracle"); }
  struct Vec {
    double v[D];
    double operator[](unsigned i) const { return v[i]; }
  };
  struct Mat {
    double v[D][D];
    const double *operator[](unsigned i) const { return v[i]; }
  };
  Vec GetOrigin() const { throw std::runtime_error("ITK stand-in: not available in the oracle"); }
  Vec GetSpacing() const { throw std::runtime_error("ITK stand-in: not available in the oracle"); }
  Mat GetDirection() const { throw std::runtime_error("ITK stand-in: not available in the oracle"); }
  template <class P, class I> bool TransformPhysicalPointToIndex(const P &, I &) const {
    throw std::runtime_error("ITK stand-in: not available in the oracle");
  }
};
}
