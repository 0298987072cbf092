// Oracle-only stand-in: the ITK major version P3MKernel.cxx selects its FFT filters by (ITK 4:
// itk::VnlForwardFFTImageFilter / itk::VnlInverseFFTImageFilter, USE_FFTWF undefined).
#pragma once
#define ITK_VERSION_MAJOR 4
