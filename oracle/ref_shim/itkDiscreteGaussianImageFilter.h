// Oracle-only stand-in: P3MKernel.cxx includes this header but uses the filter only in a comment.
#pragma once
#include "itkImage.h"
