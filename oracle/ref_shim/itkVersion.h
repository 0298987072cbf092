// Oracle-only stand-in (see itkConfigure.h).
#pragma once
#include "itkConfigure.h"
