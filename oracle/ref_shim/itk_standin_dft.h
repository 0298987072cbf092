// Oracle-only helper of the FFT filter stand-ins (itkVnlForwardFFTImageFilter.h,
// itkVnlInverseFFTImageFilter.h): the multi-dimensional discrete Fourier transform of a
// full-size complex buffer (first index fastest), computed axis by axis as direct O(n^2) sums in
// double precision, with twiddle factors exp(sign * 2 pi i (j k mod n) / n).
//   forward (sign -1): X[k] = sum_n x[n] exp(-2 pi i k.n / N)  (unnormalised)
//   inverse (sign +1): the same sum with exp(+2 pi i k.n / N); the inverse filter divides by the
//                      number of pixels, so that inverse(forward(x)) = x.
// This is the transform pair ITK's VNL FFT filters compute; only the rounding of the sums differs
// from VNL's fast transform.
#pragma once
#include <cmath>
#include <complex>
#include <vector>
namespace itk {
namespace standin {
template <unsigned D>
void dft(std::vector<std::complex<double>> &buf, const unsigned long *size, int sign) {
  const double two_pi = 6.283185307179586476925286766559;
  size_t stride = 1;
  for (unsigned ax = 0; ax < D; ++ax) {
    const size_t n = size[ax];
    size_t total = 1;
    for (unsigned i = 0; i < D; ++i) total *= size[i];
    std::vector<std::complex<double>> tw(n), line(n);
    for (size_t k = 0; k < n; ++k) {
      const double a = sign * two_pi * (double)k / (double)n;
      tw[k] = std::complex<double>(std::cos(a), std::sin(a));
    }
    const size_t outer = total / (n * stride);
    for (size_t o = 0; o < outer; ++o)
      for (size_t s = 0; s < stride; ++s) {
        const size_t base = o * n * stride + s;
        for (size_t k = 0; k < n; ++k) {
          std::complex<double> acc(0.0, 0.0);
          for (size_t j = 0; j < n; ++j) acc += buf[base + j * stride] * tw[(j * k) % n];
          line[k] = acc;
        }
        for (size_t k = 0; k < n; ++k) buf[base + k * stride] = line[k];
      }
    stride *= n;
  }
}
}  // namespace standin
}  // namespace itk
