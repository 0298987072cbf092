// Geodesic regression (the reference's Regression model, Regression.cxx) on the device: a template
// of one or several objects flows along the geodesic of (control points, initial momenta) from t0
// to tn over T time points, and each observation is matched to the template deformed to its time
// index. One iteration, replayed from a CUDA graph:
//   1. shoot and flow over [t0, tn] (Diffeos.cxx:589-712 with dt = (tn - t0) / (T - 1));
//   2. every (observation, object) data term at the observation's time index; the gradient of
//      observation s, d match / d x / (2 data_sigma2) per object (Regression.cxx:627-638);
//   3. L_data = -sum_s sum_k 0.5 match / data_sigma2 (:212-214), L_reg = -0.5 <K p, p> (:217-229);
//   4. the landmark adjoint with the observations as jumps (AdjointEquationsIntegrator.cxx:59-136)
//      and the control-point adjoint (:414-470);
//   5. dL/dp = -xi_mom(0), dL/dcp = -xi_pos(0): the reference's AddGradientRegularityTerm
//      (:676-686) takes both gradients by value, so its regularity subtractions are lost; the
//      template L2 gradient -theta(0), smoothed object by object (ConvolveGradTemplate, :688-712).
// gbk_geodesic_regression_set_corrected_gradient(1) applies the regularity gradients and adds each
// observation to the adjoint at its own time index instead (see AdjointJumps).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_deform_impl.h"
#include "gbk_dispatch.h"
#include "gbk_geometry.h"
#include "gbk_ops.h"
#include "gbk_optimize.h"
#include "gbk_registration_impl.h"

using namespace gbk;

namespace {

// L_data = sum over (observation, object) in order of -(0.5 match) / sigma2, and the sum of matches
__global__ void regression_data_kernel(const double *match, const double *sigma2, int n, double *l_data,
                                       double *match_sum) {
  pdl_entry();
  double acc = 0.0, m = 0.0;
  for (int k = 0; k < n; ++k) {
    acc -= 0.5 * match[k] / sigma2[k];
    m += match[k];
  }
  *l_data = acc;
  *match_sum = m;
}

}  // namespace

struct gbk_geodesic_regression {
  gbk_ctx *c = nullptr;
  int d = 3, T = 2, heun = 0, use_graph = 1, steps = 0, nobj = 0, nobs = 0, corrected = 0;
  long ncp = 0, nv = 0;
  double sigma_def = 1, t0 = 0, tn = 1, smoothing = 0;
  cudaStream_t stream = nullptr;
  std::vector<int> times;                  // observation time indices (increasing)
  std::vector<long> off, nvo;              // per template object: first point, point count
  std::vector<std::vector<RegObject>> obs;  // [observation][object]: data terms against the observation
  std::vector<void *> owned;
  double *cp = nullptr, *mom = nullptr, *pos = nullptr, *momt = nullptr, *lm = nullptr, *lm0 = nullptr;
  double *theta = nullptr, *xp = nullptr, *xm = nullptr, *gobs = nullptr;
  double *kp = nullptr, *greg = nullptr, *gcp = nullptr, *gmom = nullptr, *gt_l2 = nullptr, *gt_sob = nullptr;
  // out: [L, L_data, L_reg, sum of matches, <K p, p>, -, -, -, match of (observation, object) ...]
  double *out = nullptr, *sigma2 = nullptr;
  std::vector<const double *> grad_ptrs;
  DeformScratch s;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  long long graph_launches = 0;

  int alloc(void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, std::max(bytes, (size_t)8));
    if (e != cudaSuccess) return c->cuda(e, "cudaMalloc (regression)");
    owned.push_back(*p);
    return GBK_OK;
  }

  int body() {
    const long n = ncp * d, m = nv * d;
    const double span = tn - t0;
    cudaStream_t st = c->stream;
    int rc;
    if ((rc = shoot_device(c, d, ncp, cp, mom, T, sigma_def, pos, momt, s, span))) return rc;
    if ((rc = flow_device(c, d, ncp, pos, momt, T, sigma_def, nv, lm0, heun, lm, s, span))) return rc;
    for (int o = 0; o < nobs; ++o)
      for (int k = 0; k < nobj; ++k) {
        RegObject &ob = obs[o][k];
        if ((rc = ob.surf.evaluate(c, lm + (long)times[o] * m + ob.off * d, out + 8 + o * nobj + k,
                                   gobs + (long)o * m + ob.off * d, 0.5 / ob.sigma2, 0)))
          return rc;
      }
    if ((rc = c->cuda(gbk::launch(regression_data_kernel, 1, 1, 0, st, out + 8, sigma2, nobs * nobj, out + 1,
                                  out + 3),
                      "data terms")))
      return rc;
    PairArgs a = pair_args(ncp, ncp, sigma_def);
    a.x = cp;
    a.y = cp;
    a.w = mom;
    a.w_ld = d;
    a.ta = mom;
    a.ta_ld = d;
    a.out0 = kp;
    a.out0_ld = d;
    a.out1 = greg;
    a.out1_ld = d;
    if ((rc = c->launch(OP_CONV_GRADA, d, d, a))) return rc;
    if ((rc = c->cuda(dot_f64(st, kp, mom, n, out + 4, 0), "dot"))) return rc;
    if ((rc = c->cuda(scalar_combine(st, out + 2, out + 4, -0.5, nullptr, 0, nullptr, 0), "L"))) return rc;
    if ((rc = c->cuda(scalar_combine(st, out + 0, out + 1, 1.0, out + 2, 1.0, nullptr, 0), "L"))) return rc;
    c->launches += 4;
    AdjointJumps j;
    j.n = nobs;
    j.times = times.data();
    j.grads = grad_ptrs.data();
    j.reference = corrected ? 0 : 1;
    if ((rc = adjoint_landmarks_device(c, d, ncp, pos, momt, T, sigma_def, nv, lm, nullptr, heun, theta, s, span, &j)))
      return rc;
    if ((rc = adjoint_diffeo_device(c, d, ncp, pos, momt, T, sigma_def, nv, lm, theta, heun, xp, xm, s, span)))
      return rc;
    if ((rc = c->cuda(lincomb(st, gmom, nullptr, -1.0, xm, corrected ? -1.0 : 0.0, corrected ? kp : nullptr, n), "grad")))
      return rc;
    if ((rc = c->cuda(lincomb(st, gcp, nullptr, -1.0, xp, corrected ? -1.0 : 0.0, corrected ? greg : nullptr, n), "grad")))
      return rc;
    if ((rc = c->cuda(lincomb(st, gt_l2, nullptr, -1.0, theta, 0.0, nullptr, m), "grad"))) return rc;
    c->launches += 3;
    for (int k = 0; k < nobj; ++k) {  // the template gradient smoothed over each object's points
      const long o = off[k] * d;
      if (smoothing >= 1e-20) {
        PairArgs q = pair_args(nvo[k], nvo[k], smoothing);
        q.x = lm0 + o;
        q.y = lm0 + o;
        q.w = gt_l2 + o;
        q.w_ld = d;
        q.out0 = gt_sob + o;
        q.out0_ld = d;
        if ((rc = c->launch(OP_CONV, d, d, q))) return rc;
      } else {
        if ((rc = c->cuda(cudaMemcpyAsync(gt_sob + o, gt_l2 + o, (size_t)nvo[k] * d * sizeof(double),
                                          cudaMemcpyDeviceToDevice, st), "copy")))
          return rc;
      }
    }
    return GBK_OK;
  }

  int run() {
    cudaStream_t saved = c->stream;
    c->stream = stream;
    int rc = GBK_OK;
    if (!use_graph || steps == 0) {
      rc = body();
    } else {
      if (!exec) {
        if ((rc = c->cuda(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "begin capture"))) {
          c->stream = saved;
          return rc;
        }
        long long l0 = c->launches;
        rc = body();
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(stream, &g);
        if (!rc && e != cudaSuccess) rc = c->cuda(e, "end capture");
        if (!rc) rc = c->cuda(cudaGraphInstantiate(&exec, g, 0), "graph instantiate");
        graph = g;
        graph_launches = c->launches - l0;
        c->launches = l0;
      }
      if (!rc) {
        rc = c->cuda(cudaGraphLaunch(exec, stream), "graph launch");
        c->launches += graph_launches;
      }
    }
    c->stream = saved;
    if (!rc) ++steps;
    return rc;
  }

  void drop_graph() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    steps = 0;
  }

  void release() {
    drop_graph();
    for (auto &v : obs)
      for (RegObject &o : v) o.surf.release();
    for (void *p : owned) cudaFree(p);
    owned.clear();
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }
};

extern "C" {

int gbk_geodesic_regression_create(gbk_ctx *c, int d, long ncp, int nobj, const int *data_kinds, const long *nv,
                                   const double *tmpl_pts, const long *ncell, const int *tmpl_cells,
                                   const double *sigma_data, const double *data_sigma2, int nobs, const int *time_index,
                                   const long *nv_t, const double *tgt_pts, const long *ncell_t, const int *tgt_cells,
                                   int T, double sigma_def, double t0, double tn, int heun,
                                   gbk_geodesic_regression **out) {
  if (!c || !out) return GBK_ERR_ARG;
  *out = nullptr;
  c->err.clear();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "dimension %d not supported", d);
  if (nobj < 1 || nobs < 1 || ncp <= 0 || T < 2 || !(tn > t0)) return c->fail(GBK_ERR_ARG, "bad sizes");
  if (!data_kinds || !nv || !ncell || !nv_t || !ncell_t || !time_index || !sigma_data || !data_sigma2 || !tmpl_pts ||
      !tgt_pts)
    return c->fail(GBK_ERR_ARG, "null pointer");
  for (int o = 0; o < nobs; ++o) {
    if (time_index[o] < 0 || time_index[o] >= T) return c->fail(GBK_ERR_ARG, "time index %d out of range", time_index[o]);
    if (o && time_index[o] < time_index[o - 1]) return c->fail(GBK_ERR_ARG, "time indices must not decrease");
  }
  static const int term_kind[7] = {0, 1, 0, 1, 2, 2, 3};
  auto cell_of = [&](int k) { return data_kinds[k] < 2 ? 3 : data_kinds[k] < 4 ? 2 : data_kinds[k] == 5 ? d + 1 : 1; };
  for (int k = 0; k < nobj; ++k) {
    if (data_kinds[k] < 0 || data_kinds[k] > 6) return c->fail(GBK_ERR_ARG, "bad data_kind %d", data_kinds[k]);
    if (data_kinds[k] < 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "surface data terms need d = 3");
    if (!(data_sigma2[k] > 0)) return c->fail(GBK_ERR_ARG, "data_sigma2 must be positive");
    if (cell_of(k) > 1 && (!tmpl_cells || !tgt_cells)) return c->fail(GBK_ERR_ARG, "null pointer");
  }
  gbk_geodesic_regression *r = new gbk_geodesic_regression();
  r->c = c;
  r->d = d;
  r->ncp = ncp;
  r->T = T;
  r->heun = heun ? 1 : 0;
  r->sigma_def = sigma_def;
  r->t0 = t0;
  r->tn = tn;
  r->nobj = nobj;
  r->nobs = nobs;
  r->times.assign(time_index, time_index + nobs);
  for (int k = 0; k < nobj; ++k) {
    r->off.push_back(r->nv);
    r->nvo.push_back(nv[k]);
    r->nv += nv[k];
  }
  int rc = c->cuda(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking), "stream");
  // host copies of the cells (the vertex -> cell lists are built on the host)
  long tcells = 0, gcells = 0, gpts = 0;
  for (int k = 0; k < nobj; ++k)
    if (cell_of(k) > 1) tcells += ncell[k] * cell_of(k);
  for (int o = 0; o < nobs; ++o)
    for (int k = 0; k < nobj; ++k) {
      gpts += nv_t[(long)o * nobj + k];
      if (cell_of(k) > 1) gcells += ncell_t[(long)o * nobj + k] * cell_of(k);
    }
  std::vector<int> th(tcells), gh(gcells);
  if (!rc && tcells) cudaMemcpy(th.data(), tmpl_cells, th.size() * sizeof(int), cudaMemcpyDefault);
  if (!rc && gcells) cudaMemcpy(gh.data(), tgt_cells, gh.size() * sizeof(int), cudaMemcpyDefault);
  if (!rc) rc = c->cuda(cudaGetLastError(), "copy cells");
  const long n = ncp * d, m = r->nv * d, rows = std::max(ncp, r->nv);
  struct {
    double **p;
    size_t count;
  } bufs[] = {{&r->cp, (size_t)n}, {&r->mom, (size_t)n}, {&r->pos, (size_t)T * n}, {&r->momt, (size_t)T * n},
              {&r->lm, (size_t)T * m}, {&r->lm0, (size_t)m}, {&r->theta, (size_t)T * m},
              {&r->gobs, (size_t)nobs * m}, {&r->xp, (size_t)T * n}, {&r->xm, (size_t)T * n}, {&r->kp, (size_t)n},
              {&r->greg, (size_t)n}, {&r->gcp, (size_t)n}, {&r->gmom, (size_t)n}, {&r->gt_l2, (size_t)m},
              {&r->gt_sob, (size_t)m}, {&r->out, (size_t)8 + nobs * nobj}, {&r->sigma2, (size_t)nobs * nobj},
              {&r->s.va, (size_t)rows * d}, {&r->s.vb, (size_t)rows * d}, {&r->s.vc, (size_t)rows * d},
              {&r->s.vd, (size_t)rows * d}};
  for (auto &b : bufs)
    if (!rc) rc = r->alloc((void **)b.p, b.count * sizeof(double));
  if (!rc) rc = r->alloc((void **)&r->s.flag, 16);
  double *tgt = nullptr;
  if (!rc) rc = r->alloc((void **)&tgt, (size_t)std::max(gpts, 1L) * d * sizeof(double));
  cudaStream_t saved = c->stream;
  c->stream = r->stream;
  if (!rc) rc = c->cuda(cudaMemcpyAsync(tgt, tgt_pts, (size_t)gpts * d * sizeof(double), cudaMemcpyDefault, r->stream), "copy targets");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(r->lm0, tmpl_pts, (size_t)m * sizeof(double), cudaMemcpyDefault, r->stream), "copy template");
  std::vector<double> s2((size_t)nobs * nobj);
  for (int o = 0; o < nobs; ++o)
    for (int k = 0; k < nobj; ++k) s2[(size_t)o * nobj + k] = data_sigma2[k];
  if (!rc) rc = c->cuda(cudaMemcpyAsync(r->sigma2, s2.data(), s2.size() * sizeof(double), cudaMemcpyHostToDevice, r->stream), "copy");
  r->obs.resize(nobs);
  long pt_off = 0, gc_off = 0;
  for (int o = 0; o < nobs && !rc; ++o) {
    r->obs[o].resize(nobj);
    long tc_off = 0;
    for (int k = 0; k < nobj && !rc; ++k) {
      RegObject &ob = r->obs[o][k];
      const int cl = cell_of(k);
      const long vt = nv_t[(long)o * nobj + k];
      ob.off = r->off[k];
      ob.nv = nv[k];
      ob.nv_t = vt;
      ob.sigma2 = data_sigma2[k];
      const long nf = cl == 1 ? nv[k] : ncell[k], nf_t = cl == 1 ? vt : ncell_t[(long)o * nobj + k];
      rc = ob.surf.init(c, term_kind[data_kinds[k]], d, cl, sigma_data[k], nv[k], nf, cl > 1 ? th.data() + tc_off : nullptr,
                        vt, nf_t, cl > 1 ? gh.data() + gc_off : nullptr);
      if (!rc) {
        gbk_ctx::OrderScope offo(c, GBK_ORDER_TWO_FLOAT);
        rc = ob.surf.set_target(c, tgt + pt_off * d);
      }
      pt_off += vt;
      if (cl > 1) {
        tc_off += nf * cl;
        gc_off += nf_t * cl;
      }
    }
  }
  for (int o = 0; o < nobs; ++o) r->grad_ptrs.push_back(r->gobs + (long)o * m);
  if (!rc) rc = c->cuda(cudaStreamSynchronize(r->stream), "sync");
  c->stream = saved;
  if (rc) {
    r->release();
    delete r;
    return rc;
  }
  *out = r;
  return GBK_OK;
}

int gbk_geodesic_regression_set_template_smoothing(gbk_geodesic_regression *r, double width) {
  if (!r) return GBK_ERR_ARG;
  if (!(width >= 0)) return r->c->fail(GBK_ERR_ARG, "smoothing width must be >= 0");
  r->smoothing = width < 1e-20 ? 0.0 : width;
  r->drop_graph();
  return GBK_OK;
}

int gbk_geodesic_regression_set_corrected_gradient(gbk_geodesic_regression *r, int enable) {
  if (!r) return GBK_ERR_ARG;
  r->corrected = enable ? 1 : 0;
  r->drop_graph();
  return GBK_OK;
}

int gbk_geodesic_regression_set_graph(gbk_geodesic_regression *r, int enable) {
  if (!r) return GBK_ERR_ARG;
  r->use_graph = enable ? 1 : 0;
  return GBK_OK;
}

int gbk_geodesic_regression_step(gbk_geodesic_regression *r, const double *cp, const double *mom, const double *tmpl,
                                 double *loglik, double *grad_cp, double *grad_mom, double *grad_tmpl) {
  if (!r) return GBK_ERR_ARG;
  gbk_ctx *c = r->c;
  c->err.clear();
  GBK_RANGE();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (!cp || !mom) return c->fail(GBK_ERR_ARG, "null pointer");
  const size_t nb = (size_t)r->ncp * r->d * sizeof(double), mb = (size_t)r->nv * r->d * sizeof(double);
  int rc = c->cuda(cudaMemcpyAsync(r->cp, cp, nb, cudaMemcpyDefault, r->stream), "copy cp");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(r->mom, mom, nb, cudaMemcpyDefault, r->stream), "copy mom");
  if (!rc && tmpl) rc = c->cuda(cudaMemcpyAsync(r->lm0, tmpl, mb, cudaMemcpyDefault, r->stream), "copy template");
  if (!rc) {
    gbk_ctx::OrderScope off(c, GBK_ORDER_TWO_FLOAT);
    rc = r->run();
  }
  if (!rc && loglik) rc = c->cuda(cudaMemcpyAsync(loglik, r->out, 5 * sizeof(double), cudaMemcpyDefault, r->stream), "copy L");
  if (!rc && grad_cp) rc = c->cuda(cudaMemcpyAsync(grad_cp, r->gcp, nb, cudaMemcpyDefault, r->stream), "copy grad");
  if (!rc && grad_mom) rc = c->cuda(cudaMemcpyAsync(grad_mom, r->gmom, nb, cudaMemcpyDefault, r->stream), "copy grad");
  if (!rc && grad_tmpl) rc = c->cuda(cudaMemcpyAsync(grad_tmpl, r->gt_sob, mb, cudaMemcpyDefault, r->stream), "copy grad");
  if (!rc) rc = c->cuda(cudaStreamSynchronize(r->stream), "sync");
  return rc;
}

// FastGradientAscent over the reference's groups ControlPoints, InitialMomenta, TemplateData
// (alphabetical, Regression.cxx:279-286), the template step along the smoothed gradient and its
// squared norm <L2, smoothed>; Regression::SetFixedEffects (:55-66) writes the new template into
// the template objects, so every evaluation deforms its own template.
int gbk_geodesic_regression_optimize(gbk_geodesic_regression *r, double *cp, double *mom, double *tmpl,
                                     int optimize_cp, int optimize_template, int max_iterations, double initial_step,
                                     int max_line_search, double shrink, double expand, double tolerance,
                                     int nb_iter_freeze, double *history, int *iterations, double *info,
                                     double *aux_cp, double *aux_mom, double *aux_tmpl, double *grad_cp,
                                     double *grad_mom, double *grad_tmpl) {
  if (!r) return GBK_ERR_ARG;
  gbk_ctx *c = r->c;
  c->err.clear();
  GBK_RANGE();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (!cp || !mom || !tmpl || !history || !iterations) return c->fail(GBK_ERR_ARG, "null pointer");
  const long n = r->ncp * r->d, m = r->nv * r->d;
  cudaStream_t st = r->stream;
  gbk_ctx::OrderScope off(c, GBK_ORDER_TWO_FLOAT);
  double *sq_dev = nullptr;
  int rc = c->cuda(cudaMalloc(&sq_dev, 4 * sizeof(double)), "cudaMalloc (optimiser)");
  if (!rc && !optimize_cp) rc = c->cuda(cudaMemcpyAsync(r->cp, cp, n * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc && !optimize_template) rc = c->cuda(cudaMemcpyAsync(r->lm0, tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  int ng = 0, gi_cp = -1, gi_t = -1;
  long sizes[3];
  double *params[3], *aux_o[3], *grad_o[3];
  if (optimize_cp) {
    gi_cp = ng;
    sizes[ng] = n, params[ng] = cp, aux_o[ng] = aux_cp, grad_o[ng] = grad_cp;
    ++ng;
  }
  const int gi_m = ng;
  sizes[ng] = n, params[ng] = mom, aux_o[ng] = aux_mom, grad_o[ng] = grad_mom;
  ++ng;
  if (optimize_template) {
    gi_t = ng;
    sizes[ng] = m, params[ng] = tmpl, aux_o[ng] = aux_tmpl, grad_o[ng] = grad_tmpl;
    ++ng;
  }
  FgaEvaluate ev = [&](double *const *p, bool need_grad, double *terms, double *const *g, double *sq) -> int {
    int e = GBK_OK;
    if (gi_cp >= 0) e = c->cuda(cudaMemcpyAsync(r->cp, p[gi_cp], n * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
    if (!e) e = c->cuda(cudaMemcpyAsync(r->mom, p[gi_m], n * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
    if (!e && gi_t >= 0) e = c->cuda(cudaMemcpyAsync(r->lm0, p[gi_t], m * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
    if (!e) e = r->run();
    double outv[3];
    if (!e) e = c->cuda(cudaMemcpyAsync(outv, r->out, sizeof outv, cudaMemcpyDeviceToHost, st), "read L");
    double h[3] = {0, 0, 0};
    if (!e && need_grad) {
      if (gi_cp >= 0) e = c->cuda(cudaMemcpyAsync(g[gi_cp], r->gcp, n * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
      if (!e) e = c->cuda(cudaMemcpyAsync(g[gi_m], r->gmom, n * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
      if (!e && gi_t >= 0) e = c->cuda(cudaMemcpyAsync(g[gi_t], r->gt_sob, m * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
      if (!e) e = c->cuda(dot_f64(st, r->gcp, r->gcp, n, sq_dev, 0), "norm");
      if (!e) e = c->cuda(dot_f64(st, r->gmom, r->gmom, n, sq_dev + 1, 0), "norm");
      if (!e) e = c->cuda(dot_f64(st, r->gt_l2, r->gt_sob, m, sq_dev + 2, 0), "norm");
      if (!e) e = c->cuda(cudaMemcpyAsync(h, sq_dev, sizeof h, cudaMemcpyDeviceToHost, st), "read norms");
    }
    if (!e) e = c->cuda(cudaStreamSynchronize(st), "sync");
    if (!e) {
      terms[0] = outv[1];
      terms[1] = outv[2];
      if (need_grad) {
        if (gi_cp >= 0) sq[gi_cp] = h[0];
        sq[gi_m] = h[1];
        if (gi_t >= 0) sq[gi_t] = h[2];
      }
    }
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
  if (!rc) rc = fast_gradient_ascent(c, st, ng, sizes, params, o, ev, &res, aux_o, grad_o);
  // later steps use the final template
  if (!rc && optimize_template) rc = c->cuda(cudaMemcpyAsync(r->lm0, tmpl, m * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
  if (sq_dev) cudaFree(sq_dev);
  if (rc) return rc;
  std::copy(res.history.begin(), res.history.end(), history);
  *iterations = res.rows;
  if (info) {  // steps and squared norms per group (cp, momenta, template; 0 when frozen)
    for (int k = 0; k < 10; ++k) info[k] = 0.0;
    if (gi_cp >= 0) info[0] = res.step[gi_cp], info[5] = res.sq[gi_cp];
    info[1] = res.step[gi_m], info[6] = res.sq[gi_m];
    if (gi_t >= 0) info[2] = res.step[gi_t], info[7] = res.sq[gi_t];
    info[3] = res.tau;
    info[4] = res.freeze;
    info[8] = (double)res.evaluations;
    info[9] = res.stop;
  }
  return GBK_OK;
}

void gbk_geodesic_regression_destroy(gbk_geodesic_regression *r) {
  if (!r) return;
  cudaSetDevice(r->c->device);
  if (r->stream) cudaStreamSynchronize(r->stream);
  r->release();
  delete r;
}

}  // extern "C"
