// Oracle-only stand-in (see itkImage.h and itkImageRegionConstIteratorWithIndex.h).
#pragma once
#include "itkImageRegionConstIteratorWithIndex.h"
