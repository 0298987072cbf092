// Oracle-only replacement for src/support/linear_algebra/LinearAlgebra.h.
// It keeps the three Armadillo wrappers that the kernel layer uses (vector, matrix, matrix
// list) and drops the Boost-variant linear-variable wrappers, which the kernels never touch.
#pragma once
#include "ArmadilloVectorWrapper.h"
#include "ArmadilloMatrixWrapper.h"
#include "MatrixListWrapper.h"

namespace def {
namespace algebra {
typedef double ScalarType;
typedef ArmadilloVectorWrapper<ScalarType> VectorType;
typedef ArmadilloMatrixWrapper<ScalarType> MatrixType;
typedef MatrixListWrapper<ScalarType> MatrixListType;
}
}
