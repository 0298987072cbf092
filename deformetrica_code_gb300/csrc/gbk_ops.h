// Internal building blocks shared by the deformation, data-term and registration code:
// pair-kernel argument setup and the small FP64 element-wise / reduction kernels that replace the
// reference's host-side Armadillo arithmetic between kernel calls (Diffeos.cxx:627-632,
// AdjointEquationsIntegrator.cxx:117-137, OrientedSurfaceMesh.cxx:158-160, ...). Everything runs
// on the context's stream with no host synchronisation, so a whole loop can be captured in a CUDA
// graph.
#pragma once

#include <cuda_runtime.h>

#include <cstring>

#include "gbk_ctx.h"
#include "gbk_dispatch.h"

namespace gbk {

inline PairArgs pair_args(long nx, long ny, double sigma) {
  PairArgs a;
  memset(&a, 0, sizeof a);
  a.nx = nx;
  a.ny = ny;
  a.sigma = sigma < 1e-10 ? 1e-10 : sigma;
  a.nsplit = 1;
  return a;
}

// out = base + c1 * v1 + c2 * v2 over n doubles (base, v1, v2 may be null = zero). If `flag` is
// non-null and *flag != 0 (momenta below the reference's 1e-20 threshold), out = flag_value when
// given, else base.
cudaError_t lincomb(cudaStream_t st, double *out, const double *base, double c1, const double *v1,
                    double c2, const double *v2, long n, const int *flag = nullptr,
                    const double *flag_value = nullptr);

// flag = (sqrt(sum p^2) < thresh) for the n doubles of p (one CTA, FP64).
cudaError_t small_norm_flag(cudaStream_t st, const double *p, long n, double thresh, int *flag);

// *out (+)= sum_i a_i b_i in FP64 (one CTA, fixed order: bitwise reproducible).
cudaError_t dot_f64(cudaStream_t st, const double *a, const double *b, long n, double *out,
                    int accumulate);

// out = alpha * a + beta * b (scalars on the device, for assembling objectives from dots).
cudaError_t scalar_combine(cudaStream_t st, double *out, const double *a, double alpha,
                           const double *b, double beta, const double *c, double gamma);

}  // namespace gbk
