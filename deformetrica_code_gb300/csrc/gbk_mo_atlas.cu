// DeterministicAtlas with a template of one or several objects (DeformableMultiObject: surface
// meshes, polylines, point clouds, volume meshes, landmarks, each with its own data term, data
// kernel width and data sigma^2), one registration object per subject, on the device.
//
// One evaluation (DeterministicAtlas.cxx:99-154 and 200-235, AbstractAtlas.cxx:492-613):
//   per subject s, in order: copy the control points, the subject's momenta and the deformed
//   template into its registration and replay its iteration graph (shoot, flow all template
//   points, per-object data terms, regularity, adjoints);
//   L_data = sum_s L_data,s, L_reg = sum_s L_reg,s;
//   dL/dcp = sum_s dL_s/dcp, dL/dp_s = the subject's, template L2 gradient = sum_s -theta_s(0),
//   smoothed object by object over that object's points (ConvolveGradTemplate, :724-748);
//   squared norms |dL/dcp|^2, <L2, smoothed>, |dL/dp|^2 (DeterministicAtlas.cxx:230-234).
// Everything runs on the atlas's stream, subject after subject: the registrations share the
// context's scratch buffers, so their graphs must not overlap.
//
// The reference's estimator deforms a lagged template: AbstractAtlas::SetFixedEffects
// (AbstractAtlas.cxx:52-65) copies the template data it held BEFORE assigning the new fixed
// effects into the template objects, so each evaluation deforms the template of the previous
// SetFixedEffects call while the step and the smoothing use the current one. The optimiser
// reproduces that by default (gbk_mo_atlas_set_lagged_template).
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_dispatch.h"
#include "gbk_ops.h"
#include "gbk_optimize.h"
#include "gbk_registration_impl.h"

using namespace gbk;

struct gbk_mo_atlas {
  gbk_ctx *c = nullptr;
  int d = 3, nobj = 0, S = 0, lag = 1;
  long ncp = 0, nv = 0;
  double smoothing = 0.0;
  std::vector<long> off, nvo;  // per object: first template point, point count
  cudaStream_t stream = nullptr;
  std::vector<gbk_registration *> subj;
  std::vector<void *> owned;
  // the template the evaluations deform and the current fixed-effect template (lag), the L2 and
  // smoothed template gradients, scalars
  double *tmpl_def = nullptr, *tmpl_fe = nullptr, *gt_l2 = nullptr, *gt_sob = nullptr, *scal = nullptr;
  double *outs_dev = nullptr;  // S x 5 log-likelihood terms of the subjects' last runs

  int alloc(double **p, size_t n) {
    cudaError_t e = cudaMalloc(p, std::max(n, (size_t)1) * sizeof(double));
    if (e != cudaSuccess) return c->cuda(e, "cudaMalloc (atlas)");
    owned.push_back(*p);
    return GBK_OK;
  }

  std::vector<double> outs;  // the last run's log-likelihood terms per subject

  // terms[2] = {L_data, L_reg} at (cp, deformed template `moved`, mom: S x ncp x d), all device; with
  // gcp / gmom / gtmpl non-null also the gradients (the template one smoothed over the points
  // `smooth_pts`) and sq[3] = the squared norms. rerun = false: the subjects' last runs (same
  // inputs) are still in their buffers.
  int evaluate(const double *cp, const double *moved, const double *smooth_pts, const double *mom, double *terms,
               double *gcp, double *gtmpl, double *gmom, double *sq, bool rerun = true) {
    const long n = ncp * d, m = nv * d;
    const size_t nb = (size_t)n * sizeof(double);
    int rc = GBK_OK;
    outs.resize((size_t)S * 5);
    for (int s = 0; s < S && !rc && rerun; ++s) {
      gbk_registration *r = subj[s];
      rc = c->cuda(cudaMemcpyAsync(r->cp, cp, nb, cudaMemcpyDeviceToDevice, stream), "copy cp");
      if (!rc) rc = c->cuda(cudaMemcpyAsync(r->mom, mom + (long)s * n, nb, cudaMemcpyDeviceToDevice, stream), "copy mom");
      if (!rc) rc = c->cuda(cudaMemcpyAsync(r->lm0, moved, (size_t)m * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy template");
      if (!rc) rc = r->run();
      if (!rc) rc = c->cuda(cudaMemcpyAsync(outs_dev + 5 * s, r->out, 5 * sizeof(double), cudaMemcpyDeviceToDevice, stream), "gather L");
    }
    // one read of every subject's terms (a pageable read per subject would wait for each subject)
    if (!rc && rerun) rc = c->cuda(cudaMemcpyAsync(outs.data(), outs_dev, (size_t)S * 5 * sizeof(double), cudaMemcpyDeviceToHost, stream), "read L");
    const bool grad = gcp || gtmpl || gmom;
    cudaStream_t saved = c->stream;
    c->stream = stream;
    for (int s = 0; s < S && !rc && grad; ++s) {
      gbk_registration *r = subj[s];
      if (gcp) rc = c->cuda(lincomb(stream, gcp, s ? gcp : nullptr, 1.0, r->gcp, 0.0, nullptr, n), "sum grad cp");
      if (!rc && gmom) rc = c->cuda(cudaMemcpyAsync(gmom + (long)s * n, r->gmom, nb, cudaMemcpyDeviceToDevice, stream), "grad mom");
      if (!rc && gtmpl) rc = c->cuda(lincomb(stream, gt_l2, s ? gt_l2 : nullptr, -1.0, r->theta, 0.0, nullptr, m), "sum grad tmpl");
      c->launches += 2;
    }
    if (!rc && gtmpl) {
      for (int k = 0; k < nobj && !rc; ++k) {
        const long o = off[k] * d;
        if (smoothing >= 1e-20) {
          PairArgs a = pair_args(nvo[k], nvo[k], smoothing);
          a.x = smooth_pts + o;
          a.y = smooth_pts + o;
          a.w = gt_l2 + o;
          a.w_ld = d;
          a.out0 = gt_sob + o;
          a.out0_ld = d;
          rc = c->launch(OP_CONV, d, d, a);
        } else {
          rc = c->cuda(cudaMemcpyAsync(gt_sob + o, gt_l2 + o, (size_t)nvo[k] * d * sizeof(double), cudaMemcpyDeviceToDevice, stream), "copy");
        }
      }
      if (!rc) rc = c->cuda(cudaMemcpyAsync(gtmpl, gt_sob, (size_t)m * sizeof(double), cudaMemcpyDeviceToDevice, stream), "grad tmpl");
    }
    if (!rc && sq) {
      if (gcp) rc = c->cuda(dot_f64(stream, gcp, gcp, n, scal + 0, 0), "norm");
      if (!rc && gtmpl) rc = c->cuda(dot_f64(stream, gt_l2, gt_sob, m, scal + 1, 0), "norm");
      if (!rc && gmom) rc = c->cuda(dot_f64(stream, gmom, gmom, (long)S * n, scal + 2, 0), "norm");
      if (!rc) rc = c->cuda(cudaMemcpyAsync(sq, scal, 3 * sizeof(double), cudaMemcpyDeviceToHost, stream), "read norms");
      c->launches += 3;
    }
    c->stream = saved;
    if (!rc) rc = c->cuda(cudaStreamSynchronize(stream), "sync");
    if (!rc) {
      terms[0] = terms[1] = 0.0;
      for (int s = 0; s < S; ++s) {
        terms[0] += outs[5 * s + 1];
        terms[1] += outs[5 * s + 2];
      }
    }
    return rc;
  }

  void release() {
    for (gbk_registration *r : subj) {
      if (!r) continue;
      r->release();
      delete r;
    }
    subj.clear();
    for (void *p : owned) cudaFree(p);
    owned.clear();
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }
};

extern "C" {

int gbk_mo_atlas_create(gbk_ctx *c, int d, long ncp, int nobj, const int *data_kinds, const long *nv,
                        const double *tmpl_pts, const long *ncell, const int *tmpl_cells, const double *sigma_data,
                        const double *data_sigma2, int nsubj, const long *nv_t, const double *tgt_pts,
                        const long *ncell_t, const int *tgt_cells, int T, double sigma_def, int heun,
                        gbk_mo_atlas **out) {
  if (!c || !out) return GBK_ERR_ARG;
  *out = nullptr;
  c->err.clear();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (nobj < 1 || nsubj < 1 || !nv || !ncell || !nv_t || !ncell_t || !data_kinds)
    return c->fail(GBK_ERR_ARG, "bad atlas description");
  if (!tmpl_pts || !tgt_pts) return c->fail(GBK_ERR_ARG, "null pointer");
  gbk_mo_atlas *a = new gbk_mo_atlas();
  a->c = c;
  a->d = d;
  a->ncp = ncp;
  a->nobj = nobj;
  a->S = nsubj;
  for (int k = 0; k < nobj; ++k) {
    a->off.push_back(a->nv);
    a->nvo.push_back(nv[k]);
    a->nv += nv[k];
  }
  // cells per object: the registration's rule (data_kind -> vertices per cell)
  auto cell_of = [&](int k) { return data_kinds[k] < 2 ? 3 : data_kinds[k] < 4 ? 2 : data_kinds[k] == 5 ? d + 1 : 1; };
  int rc = c->cuda(cudaStreamCreateWithFlags(&a->stream, cudaStreamNonBlocking), "stream");
  long pt_off = 0, cell_off = 0;
  for (int s = 0; s < nsubj && !rc; ++s) {
    gbk_registration *r = nullptr;
    long pts = 0, cells = 0;
    for (int k = 0; k < nobj; ++k) {
      pts += nv_t[(long)s * nobj + k];
      if (cell_of(k) > 1) cells += ncell_t[(long)s * nobj + k] * cell_of(k);
    }
    rc = registration_create(c, d, ncp, nobj, data_kinds, nv, tmpl_pts, ncell, tmpl_cells, nv_t + (long)s * nobj,
                             tgt_pts + pt_off * d, ncell_t + (long)s * nobj, tgt_cells ? tgt_cells + cell_off : nullptr,
                             sigma_data, data_sigma2, T, sigma_def, heun, a->stream, &r);
    if (!rc) {
      r->pipeline = pipeline_default();  // each subject's iteration on three streams, as a registration's
      a->subj.push_back(r);
    }
    pt_off += pts;
    cell_off += cells;
  }
  const size_t m = (size_t)a->nv * d;
  if (!rc) rc = a->alloc(&a->tmpl_def, m);
  if (!rc) rc = a->alloc(&a->tmpl_fe, m);
  if (!rc) rc = a->alloc(&a->gt_l2, m);
  if (!rc) rc = a->alloc(&a->gt_sob, m);
  if (!rc) rc = a->alloc(&a->scal, 8);
  if (!rc) rc = a->alloc(&a->outs_dev, (size_t)nsubj * 5);
  if (!rc) rc = c->cuda(cudaMemcpyAsync(a->tmpl_fe, tmpl_pts, m * sizeof(double), cudaMemcpyDefault, a->stream), "copy template");
  if (!rc) rc = c->cuda(cudaStreamSynchronize(a->stream), "sync");
  if (rc) {
    a->release();
    delete a;
    return rc;
  }
  *out = a;
  return GBK_OK;
}

int gbk_mo_atlas_set_template_smoothing(gbk_mo_atlas *a, double width) {
  if (!a) return GBK_ERR_ARG;
  if (!(width >= 0)) return a->c->fail(GBK_ERR_ARG, "smoothing width must be >= 0");
  a->smoothing = width;
  return GBK_OK;
}

int gbk_mo_atlas_set_lagged_template(gbk_mo_atlas *a, int enable) {
  if (!a) return GBK_ERR_ARG;
  a->lag = enable ? 1 : 0;
  return GBK_OK;
}

int gbk_mo_atlas_step(gbk_mo_atlas *a, const double *cp, const double *tmpl, const double *mom, double *loglik,
                      double *grad_cp, double *grad_tmpl, double *grad_mom) {
  if (!a) return GBK_ERR_ARG;
  gbk_ctx *c = a->c;
  c->err.clear();
  GBK_RANGE();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (!cp || !tmpl || !mom) return c->fail(GBK_ERR_ARG, "null pointer");
  const long n = a->ncp * a->d, m = a->nv * a->d, nm = (long)a->S * n;
  // device staging: cp, template, momenta, and the three gradients
  std::vector<double *> buf(6, nullptr);
  const long sizes[6] = {n, m, nm, n, m, nm};
  int rc = GBK_OK;
  for (int i = 0; i < 6 && !rc; ++i) rc = c->cuda(cudaMalloc(&buf[i], sizes[i] * sizeof(double)), "cudaMalloc (atlas step)");
  cudaStream_t st = a->stream;
  if (!rc) rc = c->cuda(cudaMemcpyAsync(buf[0], cp, n * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(buf[1], tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(buf[2], mom, nm * sizeof(double), cudaMemcpyDefault, st), "copy");
  double terms[2] = {0, 0};
  if (!rc) {
    gbk_ctx::OrderScope off(c, GBK_ORDER_TWO_FLOAT);
    rc = a->evaluate(buf[0], buf[1], buf[1], buf[2], terms, grad_cp ? buf[3] : nullptr, grad_tmpl ? buf[4] : nullptr,
                     grad_mom ? buf[5] : nullptr, nullptr);
  }
  if (!rc && grad_cp) rc = c->cuda(cudaMemcpyAsync(grad_cp, buf[3], n * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc && grad_tmpl) rc = c->cuda(cudaMemcpyAsync(grad_tmpl, buf[4], m * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc && grad_mom) rc = c->cuda(cudaMemcpyAsync(grad_mom, buf[5], nm * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
  cudaStreamSynchronize(st);
  for (double *p : buf)
    if (p) cudaFree(p);
  if (!rc && loglik) {
    loglik[0] = terms[0] + terms[1];
    loglik[1] = terms[0];
    loglik[2] = terms[1];
  }
  return rc;
}

int gbk_mo_atlas_optimize(gbk_mo_atlas *a, double *cp, double *tmpl, double *mom, int optimize_cp,
                          int optimize_template, int max_iterations, double initial_step, int max_line_search,
                          double shrink, double expand, double tolerance, int nb_iter_freeze, double *history,
                          int *iterations, double *info, double *aux_cp, double *aux_tmpl, double *aux_mom,
                          double *grad_cp, double *grad_tmpl, double *grad_mom) {
  if (!a) return GBK_ERR_ARG;
  gbk_ctx *c = a->c;
  c->err.clear();
  GBK_RANGE();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (!cp || !tmpl || !mom || !history || !iterations) return c->fail(GBK_ERR_ARG, "null pointer");
  const long n = a->ncp * a->d, m = a->nv * a->d, nm = (long)a->S * n;
  cudaStream_t st = a->stream;
  gbk_ctx::OrderScope off(c, GBK_ORDER_TWO_FLOAT);
  // frozen groups live in device copies; groups in the reference's order [cp] [template] momenta
  double *cp_frozen = nullptr, *tmpl_frozen = nullptr;
  int rc = GBK_OK;
  if (!optimize_cp) rc = c->cuda(cudaMalloc(&cp_frozen, n * sizeof(double)), "cudaMalloc");
  if (!rc && !optimize_template) rc = c->cuda(cudaMalloc(&tmpl_frozen, m * sizeof(double)), "cudaMalloc");
  if (!rc && cp_frozen) rc = c->cuda(cudaMemcpyAsync(cp_frozen, cp, n * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc && tmpl_frozen) rc = c->cuda(cudaMemcpyAsync(tmpl_frozen, tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  // the deformed and the current template start at the initial one
  if (!rc) rc = c->cuda(cudaMemcpyAsync(a->tmpl_fe, tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(a->tmpl_def, tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  int ng = 0, gi_cp = -1, gi_t = -1;
  long sizes[3];
  double *params[3], *aux_o[3], *grad_o[3];
  if (optimize_cp) {
    gi_cp = ng;
    sizes[ng] = n, params[ng] = cp, aux_o[ng] = aux_cp, grad_o[ng] = grad_cp;
    ++ng;
  }
  if (optimize_template) {
    gi_t = ng;
    sizes[ng] = m, params[ng] = tmpl, aux_o[ng] = aux_tmpl, grad_o[ng] = grad_tmpl;
    ++ng;
  }
  const int gi_m = ng;
  sizes[ng] = nm, params[ng] = mom, aux_o[ng] = aux_mom, grad_o[ng] = grad_mom;
  ++ng;
  const bool lag = a->lag && optimize_template;
  // With the lag the ascent evaluates the extrapolated point twice in a row, the log-likelihood and
  // then the gradient, with only SetFixedEffects calls between (which write no parameter buffer);
  // the second evaluation reuses the subjects' runs when the parameter buffers and the buffer the
  // deformed template was copied from are the same.
  const double *fe_src = tmpl, *def_src = tmpl;
  const double *last_p[3] = {nullptr, nullptr, nullptr}, *last_def = nullptr;
  bool last_nograd = false;
  FgaEvaluate ev = [&](double *const *p, bool need_grad, double *terms, double *const *g, double *sq) -> int {
    const double *pcp = optimize_cp ? p[gi_cp] : cp_frozen;
    const double *pt = optimize_template ? p[gi_t] : tmpl_frozen;
    bool reuse = lag && need_grad && last_nograd && def_src == last_def;
    for (int k = 0; k < ng; ++k) reuse = reuse && last_p[k] == p[k];
    for (int k = 0; k < ng; ++k) last_p[k] = p[k];
    last_def = def_src;
    last_nograd = !need_grad;
    double h[3] = {0, 0, 0};
    int e = a->evaluate(pcp, lag ? a->tmpl_def : pt, pt, p[gi_m], terms, need_grad && optimize_cp ? g[gi_cp] : nullptr,
                        need_grad && optimize_template ? g[gi_t] : nullptr, need_grad ? g[gi_m] : nullptr,
                        need_grad ? h : nullptr, !reuse);
    if (!e && need_grad) {
      if (optimize_cp) sq[gi_cp] = h[0];
      if (optimize_template) sq[gi_t] = h[1];
      sq[gi_m] = h[2];
    }
    return e;
  };
  // SetFixedEffects: the template objects take the previous fixed-effect template
  FgaSetFixed sf = [&](double *const *p) -> int {
    def_src = fe_src;
    fe_src = p[gi_t];
    int e = c->cuda(cudaMemcpyAsync(a->tmpl_def, a->tmpl_fe, m * sizeof(double), cudaMemcpyDeviceToDevice, st), "lag");
    if (!e) e = c->cuda(cudaMemcpyAsync(a->tmpl_fe, p[gi_t], m * sizeof(double), cudaMemcpyDeviceToDevice, st), "lag");
    return e;
  };
  FgaOptions o;
  o.estimator = c->estimator;
  o.max_iterations = max_iterations;
  o.max_line_search = max_line_search;
  o.nb_iter_freeze = nb_iter_freeze;
  o.initial_step = initial_step;
  o.shrink = shrink;
  o.expand = expand;
  o.tolerance = tolerance;
  FgaResult res;
  if (!rc) rc = fast_gradient_ascent(c, st, ng, sizes, params, o, ev, &res, aux_o, grad_o, lag ? sf : FgaSetFixed());
  cudaStreamSynchronize(st);
  if (cp_frozen) cudaFree(cp_frozen);
  if (tmpl_frozen) cudaFree(tmpl_frozen);
  if (rc) return rc;
  std::copy(res.history.begin(), res.history.end(), history);
  *iterations = res.rows;
  if (info) {
    info[0] = optimize_cp ? res.step[gi_cp] : 0.0;
    info[1] = optimize_template ? res.step[gi_t] : 0.0;
    info[2] = res.step[gi_m];
    info[3] = res.tau;
    info[4] = res.freeze;
    info[5] = optimize_cp ? res.sq[gi_cp] : 0.0;
    info[6] = optimize_template ? res.sq[gi_t] : 0.0;
    info[7] = res.sq[gi_m];
    info[8] = (double)res.evaluations;
    info[9] = res.stop;
  }
  return GBK_OK;
}

void gbk_mo_atlas_destroy(gbk_mo_atlas *a) {
  if (!a) return;
  cudaSetDevice(a->c->device);
  if (a->stream) cudaStreamSynchronize(a->stream);
  a->release();
  delete a;
}

}  // extern "C"
