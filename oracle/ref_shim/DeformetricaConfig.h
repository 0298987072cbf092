// Build configuration for compiling the reference kernel layer as the FP64 oracle.
// The reference hard-defines double precision; the CUDA and fast-math paths stay off.
#pragma once
#define DEFORMETRICA_CONFIG
#define USE_DOUBLE_PRECISION
