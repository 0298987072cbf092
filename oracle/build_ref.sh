#!/usr/bin/env bash
# Builds the reference's own FP64 kernel layer into oracle/_ref/libref_exactkernel.so.
#
# Compiles, in place and unmodified, the reference sources
#   src/support/kernels/ExactKernel.cxx, src/support/kernels/AbstractKernel.cxx,
#   src/support/kernels/P3MKernel.cxx,
#   src/support/linear_algebra/Armadillo{Matrix,Vector}Wrapper.cxx, MatrixListWrapper.cxx,
#   src/support/utilities/SimpleTimer.cxx
# against the vendored, header-only Armadillo 7.700 (extra/armadillo-7.700.0.tar.xz, extracted
# into oracle/_ref/) and the small stand-in headers in oracle/ref_shim/, with the reference's
# RELEASE optimisation level (-O2). Nothing is copied out of the reference tree; all outputs go
# to oracle/_ref/. Usage: oracle/build_ref.sh [REFERENCE_ROOT]  (default: $DEFORMETRICA_REFERENCE_DIR,
# else the checkout location of this build's container, /root/reference).
set -euo pipefail
REF="${1:-${DEFORMETRICA_REFERENCE_DIR:-/root/reference}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
if [ ! -d "$REF/src/support/kernels" ]; then
  echo "build_ref.sh: reference tree not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT"
ARMA="$OUT/armadillo-7.700.0"
if [ ! -f "$ARMA/include/armadillo" ]; then
  tar -xJf "$REF/extra/armadillo-7.700.0.tar.xz" -C "$OUT"
fi
S="$REF/src/support"
CXXFLAGS=(-std=c++14 -O2 -fPIC -w
  -DARMA_DONT_USE_WRAPPER -DARMA_DONT_USE_LAPACK -DARMA_DONT_USE_BLAS -DARMA_DONT_USE_HDF5
  -I"$HERE/ref_shim" -I"$S/kernels" -I"$S/linear_algebra" -I"$S/utilities" -I"$S/fast_math"
  -I"$ARMA/include")
SRCS=("$HERE/ref_driver.cpp" "$S/kernels/ExactKernel.cxx" "$S/kernels/AbstractKernel.cxx" "$S/kernels/P3MKernel.cxx"
  "$S/linear_algebra/ArmadilloMatrixWrapper.cxx" "$S/linear_algebra/ArmadilloVectorWrapper.cxx"
  "$S/linear_algebra/MatrixListWrapper.cxx" "$S/utilities/SimpleTimer.cxx")
OBJS=()
for s in "${SRCS[@]}"; do
  o="$OUT/$(basename "${s%.*}").o"
  g++ "${CXXFLAGS[@]}" -c "$s" -o "$o" &
  OBJS+=("$o")
done
wait
g++ -shared -o "$OUT/libref_exactkernel.so" "${OBJS[@]}"
echo "$OUT/libref_exactkernel.so"
