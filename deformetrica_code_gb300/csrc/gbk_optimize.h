// Device-resident FastGradientAscent (FastGradientAscent.cxx:48-335) and GradientAscent
// (GradientAscent.cxx:48-240) over groups of device vectors: the host takes the line-search
// decisions from a few scalars per evaluation, every parameter, trial point and gradient stays in
// device memory. Used by the registration, atlas and regression optimisers.
#pragma once

#include <cuda_runtime.h>

#include <functional>
#include <vector>

struct gbk_ctx;

namespace gbk {

struct FgaOptions {
  int estimator = 0;  // GBK_ESTIMATOR_FAST_GRADIENT_ASCENT or GBK_ESTIMATOR_GRADIENT_ASCENT
  int max_iterations = 10;
  int max_line_search = 10;
  int nb_iter_freeze = 3;
  double initial_step = 1e-3;
  double shrink = 0.5;
  double expand = 1.2;
  double tolerance = 1e-4;
};

struct FgaResult {
  std::vector<double> history;  // rows x 2: [data, regularity] per accepted iteration
  int rows = 0;
  std::vector<double> step, sq;  // per group: final step size, squared gradient norm
  double tau = 1.0;
  int freeze = 1;
  long evaluations = 0;
  int stop = 0;  // 0 max iterations, 1 line search exhausted, 2 tolerance
  int iter = 0;  // the estimator's iteration counter at the end (the state's "iter")
};

// evaluate(params, need_grad, terms, grads, sq): the log-likelihood terms [data, regularity] at
// `params` (one device vector per group) into terms; with need_grad also the gradient of every
// group into grads (device) and the squared norm the step is weighted with into sq (host).
typedef std::function<int(double *const *params, bool need_grad, double *terms, double *const *grads, double *sq)>
    FgaEvaluate;

// set_fixed(params): called wherever the reference calls SetFixedEffects (before every evaluation
// at a new point and around the per-iteration state write), for models whose state depends on that
// sequence; with it the log-likelihood at the extrapolated point and the gradient there are two
// evaluations, as in FastGradientAscent.cxx:245-258.
typedef std::function<int(double *const *params)> FgaSetFixed;

// Runs the ascent (o.estimator) from the group vectors `params` (device, sizes[g] doubles each),
// which receive the final fixed effects; aux_out / grad_out (optional, device or host, per group)
// receive the extrapolated point (FastGradientAscent; GradientAscent has none and leaves aux_out
// untouched) and the last gradient.
int fast_gradient_ascent(gbk_ctx *c, cudaStream_t st, int ng, const long *sizes, double *const *params,
                         const FgaOptions &o, const FgaEvaluate &evaluate, FgaResult *res, double *const *aux_out,
                         double *const *grad_out, const FgaSetFixed &set_fixed = nullptr);

}  // namespace gbk
