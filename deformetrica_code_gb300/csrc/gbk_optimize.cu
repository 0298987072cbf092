// FastGradientAscent::Update (FastGradientAscent.cxx:48-300) and GradientAscentStep (:306-335)
// over groups of device vectors. Steps, in the reference's order:
//   start: evaluate at the start point with gradients; history[0]; step = initial step per group;
//   each iteration: line search from the extrapolated point aux along the gradient there,
//     new = aux + grad * step; accept if L(new) - L(aux) - <sq, step> shrink >= 0 (counting the
//     accepted-at-once streak); otherwise shrink every step and, with several groups, also try
//     each "all but one shrunk" proposal and keep the best acceptable one (multivariate line
//     search); a single group just shrinks;
//   after an accepted step: tau' = (1 + sqrt(1 + 4 tau^2)) / 2, expanding the steps (and using
//     tau^2 / expand) once the streak exceeds nb_iter_freeze; aux = new + (new - fixed)(tau - 1)
//     / tau'; fixed = new; evaluate at aux with gradients; stop when the last change of L is below
//     tolerance times the change since the start.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_ops.h"
#include "gbk_optimize.h"

namespace gbk {

// GradientAscent::Update (GradientAscent.cxx:48-240): the trial fixed + grad * step is accepted when
// the log-likelihood does not decrease; otherwise every step shrinks and, with several groups,
// each "all but one shrunk" proposal is tried and the best acceptable one kept (its step
// restored); after an accepted step every step expands, the tolerance is tested, and the gradient
// is evaluated at the new fixed point (after SetFixedEffects, as the reference).
static int gradient_ascent(gbk_ctx *c, cudaStream_t st, int ng, const long *sizes, double *const *params,
                           const FgaOptions &o, const FgaEvaluate &evaluate, FgaResult *res,
                           double *const *grad_out, const FgaSetFixed &set_fixed) {
  std::vector<double *> owned;
  auto dev = [&](long n, double **p) {
    int e = c->cuda(cudaMalloc(p, (size_t)std::max(n, 1L) * sizeof(double)), "cudaMalloc (optimiser)");
    if (!e) owned.push_back(*p);
    return e;
  };
  std::vector<double *> fixed(ng), nw(ng), grad(ng);
  std::vector<std::vector<double *>> prop(ng, std::vector<double *>(ng));
  int rc = GBK_OK;
  for (int g = 0; g < ng && !rc; ++g) {
    if (!rc) rc = dev(sizes[g], &fixed[g]);
    if (!rc) rc = dev(sizes[g], &nw[g]);
    if (!rc) rc = dev(sizes[g], &grad[g]);
    for (int k = 0; k < ng && !rc; ++k) rc = dev(sizes[g], &prop[k][g]);
  }
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    for (double *p : owned) cudaFree(p);
  };
  if (rc) {
    cleanup();
    return rc;
  }
  const double shrink = o.shrink;
  std::vector<double> sq(ng, 0.0), step(ng, o.initial_step), hist((size_t)(o.max_iterations + 1) * 2, 0.0);
  long evaluations = 0;
  auto eval = [&](const std::vector<double *> &p, bool need_grad, double *t) {
    ++evaluations;
    return evaluate(p.data(), need_grad, t, grad.data(), sq.data());
  };
  auto setf = [&](const std::vector<double *> &p) { return set_fixed ? set_fixed(p.data()) : GBK_OK; };
  auto ascent = [&](const std::vector<double *> &dst, const std::vector<double> &s) {
    int e = GBK_OK;
    for (int g = 0; g < ng && !e; ++g) e = c->cuda(lincomb(st, dst[g], fixed[g], s[g], grad[g], 0.0, nullptr, sizes[g]), "ascent");
    return e;
  };
  for (int g = 0; g < ng && !rc; ++g)
    rc = c->cuda(cudaMemcpyAsync(fixed[g], params[g], (size_t)sizes[g] * sizeof(double), cudaMemcpyDefault, st), "copy");
  double t0[2] = {0, 0}, ignored[2];
  if (!rc) rc = eval(fixed, false, t0);
  if (!rc) rc = eval(fixed, true, ignored);
  if (rc) {
    cleanup();
    return rc;
  }
  hist[0] = t0[0];
  hist[1] = t0[1];
  double lsq_ref = t0[0] + t0[1];
  int it = 1, stop = 0, rows = 0;
  while (it < o.max_iterations + 1 && !rc) {
    bool found = false;
    double new_terms[2] = {0, 0};
    for (int li = 0; li < o.max_line_search && !rc; ++li) {
      double t[2];
      if ((rc = ascent(nw, step))) break;
      if ((rc = setf(nw))) break;
      if ((rc = eval(nw, false, t))) break;
      if (t[0] + t[1] - lsq_ref >= 0) {
        found = true;
        new_terms[0] = t[0];
        new_terms[1] = t[1];
        break;
      } else if (ng > 1) {
        for (int g = 0; g < ng; ++g) step[g] *= shrink;
        std::vector<double> qs(ng);
        std::vector<std::array<double, 2>> ts(ng);
        for (int k = 0; k < ng && !rc; ++k) {
          std::vector<double> local(step);
          local[k] /= shrink;
          if ((rc = ascent(prop[k], local))) break;
          if ((rc = setf(prop[k]))) break;
          if ((rc = eval(prop[k], false, ts[k].data()))) break;
          qs[k] = ts[k][0] + ts[k][1] - lsq_ref;
        }
        if (rc) break;
        int idx = 0;
        for (int k = 1; k < ng; ++k)
          if (qs[k] > qs[idx]) idx = k;
        if (qs[idx] >= 0) {
          std::swap(nw, prop[idx]);
          new_terms[0] = ts[idx][0];
          new_terms[1] = ts[idx][1];
          step[idx] /= shrink;
          found = true;
          break;
        }
      } else {
        for (int g = 0; g < ng; ++g) step[g] *= shrink;
      }
    }
    if (rc) break;
    if (!found) {
      rc = setf(fixed);
      stop = 1;
      rows = it;
      break;
    }
    hist[(size_t)it * 2] = new_terms[0];
    hist[(size_t)it * 2 + 1] = new_terms[1];
    std::swap(fixed, nw);
    for (int g = 0; g < ng; ++g) step[g] *= o.expand;
    lsq_ref = new_terms[0] + new_terms[1];
    const double cur = (hist[(size_t)(it - 1) * 2] + hist[(size_t)(it - 1) * 2 + 1]) -
                       (hist[(size_t)it * 2] + hist[(size_t)it * 2 + 1]);
    const double ref = (hist[0] + hist[1]) - (hist[(size_t)it * 2] + hist[(size_t)it * 2 + 1]);
    if (std::fabs(cur) < o.tolerance * std::fabs(ref)) {
      stop = 2;
      rows = it + 1;
      break;
    }
    if ((rc = setf(fixed))) break;
    if ((rc = eval(fixed, true, ignored))) break;
    ++it;
    rows = it;
  }
  for (int g = 0; g < ng && !rc; ++g) {
    const size_t nb = (size_t)sizes[g] * sizeof(double);
    rc = c->cuda(cudaMemcpyAsync(params[g], fixed[g], nb, cudaMemcpyDefault, st), "copy");
    if (!rc && grad_out && grad_out[g]) rc = c->cuda(cudaMemcpyAsync(grad_out[g], grad[g], nb, cudaMemcpyDefault, st), "copy");
  }
  if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
  if (!rc) {
    res->rows = stop == 0 ? o.max_iterations + 1 : rows;
    res->history.assign(hist.begin(), hist.begin() + (size_t)res->rows * 2);
    res->step = step;
    res->sq = sq;
    res->tau = 0.0;
    res->freeze = 0;
    res->evaluations = evaluations;
    res->stop = stop;
    res->iter = it;
  }
  cleanup();
  return rc;
}

int fast_gradient_ascent(gbk_ctx *c, cudaStream_t st, int ng, const long *sizes, double *const *params,
                         const FgaOptions &o, const FgaEvaluate &evaluate, FgaResult *res, double *const *aux_out,
                         double *const *grad_out, const FgaSetFixed &set_fixed) {
  if (ng < 1 || ng > 4) return c->fail(GBK_ERR_ARG, "optimiser: %d parameter groups", ng);
  if (o.max_iterations < 0 || o.max_line_search < 1 || !(o.shrink > 0 && o.shrink < 1) || !(o.expand >= 1) ||
      !(o.initial_step > 0) || o.nb_iter_freeze < 0)
    return c->fail(GBK_ERR_ARG, "bad optimiser parameters");
  if (o.estimator == GBK_ESTIMATOR_GRADIENT_ASCENT)
    return gradient_ascent(c, st, ng, sizes, params, o, evaluate, res, grad_out, set_fixed);
  if (o.estimator != GBK_ESTIMATOR_FAST_GRADIENT_ASCENT) return c->fail(GBK_ERR_ARG, "unknown estimator %d", o.estimator);
  // per group: fixed, aux, new, gradient, and one candidate per multivariate proposal
  std::vector<double *> owned;
  auto dev = [&](long n, double **p) {
    int e = c->cuda(cudaMalloc(p, (size_t)std::max(n, 1L) * sizeof(double)), "cudaMalloc (optimiser)");
    if (!e) owned.push_back(*p);
    return e;
  };
  std::vector<double *> fixed(ng), aux(ng), nw(ng), grad(ng);
  std::vector<std::vector<double *>> prop(ng, std::vector<double *>(ng));
  int rc = GBK_OK;
  for (int g = 0; g < ng && !rc; ++g) {
    if (!rc) rc = dev(sizes[g], &fixed[g]);
    if (!rc) rc = dev(sizes[g], &aux[g]);
    if (!rc) rc = dev(sizes[g], &nw[g]);
    if (!rc) rc = dev(sizes[g], &grad[g]);
    for (int k = 0; k < ng && !rc; ++k) rc = dev(sizes[g], &prop[k][g]);
  }
  auto cleanup = [&]() {
    cudaStreamSynchronize(st);
    for (double *p : owned) cudaFree(p);
  };
  if (rc) {
    cleanup();
    return rc;
  }
  const double shrink = o.shrink;
  std::vector<double> sq(ng, 0.0), step(ng, o.initial_step), hist((size_t)(o.max_iterations + 1) * 2, 0.0);
  long evaluations = 0;
  auto eval = [&](const std::vector<double *> &p, bool need_grad, double *t) {
    ++evaluations;
    return evaluate(p.data(), need_grad, t, grad.data(), sq.data());
  };
  auto setf = [&](const std::vector<double *> &p) { return set_fixed ? set_fixed(p.data()) : GBK_OK; };
  // the log-likelihood at aux and the gradient there: one evaluation, or, with set_fixed, the
  // reference's sequence (evaluate; SetFixedEffects(fixed) and (aux) for the state write; gradient)
  auto eval_aux = [&](double *t, bool after_step) {
    if (!set_fixed) return eval(aux, true, t);
    int e = after_step ? setf(aux) : GBK_OK;
    if (!e) e = eval(aux, false, t);
    if (!e && after_step) e = setf(fixed);
    if (!e && after_step) e = setf(aux);
    double ignored[2];
    if (!e) e = eval(aux, true, ignored);
    if (!e) --evaluations;  // one log-likelihood evaluation and one gradient
    return e;
  };
  auto ascent = [&](const std::vector<double *> &dst, const std::vector<double> &s) {  // GradientAscentStep
    int e = GBK_OK;
    for (int g = 0; g < ng && !e; ++g) e = c->cuda(lincomb(st, dst[g], aux[g], s[g], grad[g], 0.0, nullptr, sizes[g]), "ascent");
    return e;
  };
  auto dotsq = [&](const std::vector<double> &s) {
    double v = 0.0;
    for (int g = 0; g < ng; ++g) v += sq[g] * s[g];
    return v;
  };
  for (int g = 0; g < ng && !rc; ++g) {
    rc = c->cuda(cudaMemcpyAsync(fixed[g], params[g], (size_t)sizes[g] * sizeof(double), cudaMemcpyDefault, st), "copy");
    if (!rc) rc = c->cuda(cudaMemcpyAsync(aux[g], params[g], (size_t)sizes[g] * sizeof(double), cudaMemcpyDefault, st), "copy");
  }
  double t0[2] = {0, 0};
  if (!rc) rc = eval_aux(t0, false);
  if (rc) {
    cleanup();
    return rc;
  }
  hist[0] = t0[0];
  hist[1] = t0[1];
  double lsq_ref = t0[0] + t0[1];
  double tau = 1.0;
  int freeze = 1, it = 1, stop = 0;
  while (it < o.max_iterations + 1 && !rc) {
    bool found = false;
    double new_terms[2] = {0, 0};
    for (int li = 0; li < o.max_line_search && !rc; ++li) {
      double t[2];
      if ((rc = ascent(nw, step))) break;
      if ((rc = setf(nw))) break;
      if ((rc = eval(nw, false, t))) break;
      if (t[0] + t[1] - lsq_ref - dotsq(step) * shrink >= 0) {
        found = true;
        new_terms[0] = t[0];
        new_terms[1] = t[1];
        if (li == 0) ++freeze;
        break;
      } else if (ng > 1) {  // every group but one shrunk, all configurations tried
        freeze = 1;
        for (int g = 0; g < ng; ++g) step[g] *= shrink;
        std::vector<double> qs(ng);
        std::vector<std::array<double, 2>> ts(ng);
        for (int k = 0; k < ng && !rc; ++k) {
          std::vector<double> local(step);
          local[k] /= shrink;
          if ((rc = ascent(prop[k], local))) break;
          if ((rc = setf(prop[k]))) break;
          if ((rc = eval(prop[k], false, ts[k].data()))) break;
          qs[k] = ts[k][0] + ts[k][1] - lsq_ref - dotsq(local) * shrink;
        }
        if (rc) break;
        int idx = 0;
        for (int k = 1; k < ng; ++k)
          if (qs[k] > qs[idx]) idx = k;
        if (qs[idx] >= 0) {
          std::swap(nw, prop[idx]);
          new_terms[0] = ts[idx][0];
          new_terms[1] = ts[idx][1];
          step[idx] /= shrink;
          found = true;
          break;
        }
      } else {
        freeze = 1;
        for (int g = 0; g < ng; ++g) step[g] *= shrink;
      }
    }
    if (rc) break;
    if (!found) {
      rc = setf(fixed);
      stop = 1;
      break;
    }
    hist[(size_t)it * 2] = new_terms[0];
    hist[(size_t)it * 2 + 1] = new_terms[1];
    double tau_next = (1.0 + std::sqrt(1.0 + 4.0 * tau * tau)) / 2.0;
    if (freeze > o.nb_iter_freeze) {
      for (int g = 0; g < ng; ++g) step[g] *= o.expand;
      tau_next = (1.0 + std::sqrt(1.0 + 4.0 * tau * tau / o.expand)) / 2.0;
    }
    const double ts_ = (tau - 1.0) / tau_next;
    for (int g = 0; g < ng && !rc; ++g)
      rc = c->cuda(lincomb(st, aux[g], nw[g], ts_, nw[g], -ts_, fixed[g], sizes[g]), "extrapolate");
    if (rc) break;
    std::swap(fixed, nw);
    tau = tau_next;
    double ta[2];
    if ((rc = eval_aux(ta, true))) break;
    lsq_ref = ta[0] + ta[1];
    const double cur = (hist[(size_t)(it - 1) * 2] + hist[(size_t)(it - 1) * 2 + 1]) -
                       (hist[(size_t)it * 2] + hist[(size_t)it * 2 + 1]);
    const double ref = (hist[0] + hist[1]) - (hist[(size_t)it * 2] + hist[(size_t)it * 2 + 1]);
    ++it;
    if (std::fabs(cur) < o.tolerance * std::fabs(ref)) {
      stop = 2;
      break;
    }
  }
  if (!rc) rc = setf(fixed);
  for (int g = 0; g < ng && !rc; ++g) {
    const size_t nb = (size_t)sizes[g] * sizeof(double);
    rc = c->cuda(cudaMemcpyAsync(params[g], fixed[g], nb, cudaMemcpyDefault, st), "copy");
    if (!rc && aux_out && aux_out[g]) rc = c->cuda(cudaMemcpyAsync(aux_out[g], aux[g], nb, cudaMemcpyDefault, st), "copy");
    if (!rc && grad_out && grad_out[g]) rc = c->cuda(cudaMemcpyAsync(grad_out[g], grad[g], nb, cudaMemcpyDefault, st), "copy");
  }
  if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
  if (!rc) {
    res->rows = stop == 1 ? it : std::min(it, o.max_iterations + 1);
    res->history.assign(hist.begin(), hist.begin() + (size_t)res->rows * 2);
    res->step = step;
    res->sq = sq;
    res->tau = tau;
    res->freeze = freeze;
    res->evaluations = evaluations;
    res->stop = stop;
    res->iter = it;
  }
  cleanup();
  return rc;
}

}  // namespace gbk
