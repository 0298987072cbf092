// Oracle-only stand-in (see itkImage.h).
#pragma once
#include "itkImage.h"
