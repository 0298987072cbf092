// One registration iteration of a subject of DeterministicAtlas with a frozen template of one or
// several objects (triangle meshes, polylines, point clouds, volume meshes, landmarks), on the
// device, replayed from a CUDA graph.
//
// Log-likelihood (DeterministicAtlas.cxx:99-154) L = -0.5 sum_k match_k / data_sigma2_k
// - 0.5 <K p, p>
// and its gradient (AbstractAtlas.cxx:559-613, DeterministicAtlas.cxx:246-280):
//   1. Shoot the control points and momenta (Diffeos.cxx:589-660);
//   2. flow the template vertices (Diffeos.cxx:661-712);
//   3. the data term and its vertex gradient (currents or varifold), seeding the landmark adjoint
//      with grad / (2 data_sigma2) (AbstractAtlas.cxx:585-590);
//   4. the RKHS regularity <K p, p> and its gradients K p and ConvolveGradient(cp, p);
//   5. the landmark and diffeomorphism-parameter adjoints (AdjointEquationsIntegrator.cxx:33-570);
//   6. dL/dp = -xi_mom(0) - K p, dL/dcp = -xi_pos(0) - ConvolveGradient(cp, p).
// Every buffer is allocated at creation, the first step runs eagerly (sizing the context's split
// buffer), the second step is captured into a CUDA graph and later steps replay the graph: one
// graph launch per iteration, no allocation and no host synchronisation inside it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_deform_impl.h"
#include "gbk_dispatch.h"
#include "gbk_geometry.h"
#include "gbk_hostio.h"
#include "gbk_ops.h"
#include "gbk_optimize.h"
#include "gbk_registration_impl.h"

using namespace gbk;

namespace gbk {
int pipeline_default() {
  const char *e = getenv("GBK_PIPELINE");
  return e && e[0] == '0' ? 0 : 1;
}
}  // namespace gbk

namespace {

// L_data = 0.5 * (-sum_k match_k / sigma2_k) in object order (DeterministicAtlas.cxx:121-125) and
// the sum of the matches
__global__ void data_terms_kernel(const double *match, const double *sigma2, int n, double *l_data,
                                  double *match_sum) {
  pdl_entry();
  double acc = 0.0, m = 0.0;
  for (int k = 0; k < n; ++k) {
    acc -= match[k] / sigma2[k];
    m += match[k];
  }
  *l_data = acc * 0.5;
  *match_sum = m;
}

}  // namespace

int gbk_registration::alloc(void **p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, std::max(bytes, (size_t)8));
  if (e != cudaSuccess) return c->cuda(e, "cudaMalloc (registration)");
  owned.push_back(*p);
  return GBK_OK;
}

// Helper context, second scratch set and events of the pipelined iteration (once per registration).
int gbk_registration::enable_pipeline() {
  if (c2) return GBK_OK;
  int rc = GBK_OK;
  gbk_ctx **helpers[2] = {&c2, &c3};
  unsigned long long **words[2] = {&c2_words, &c3_words};
  for (int k = 0; k < 2 && !rc; ++k) {
    gbk_ctx *h = nullptr;
    if (gbk_create(c->device, &h) != GBK_OK) {
      rc = c->fail(GBK_ERR_CUDA, "pipelined registration: helper context: %s", gbk_last_error(nullptr));
      break;
    }
    // the helper's kernel sums count into this context's pair counters and report into its status
    // word; its own words stay allocated (its spatial order would use them) and are restored on release
    *helpers[k] = h;
    *words[k] = h->pair_counter;
    h->pair_counter = c->pair_counter;
    h->status = c->status;
  }
  const long rows = std::max(ncp, nv);
  double **bufs[] = {&s2.va, &s2.vb, &s2.vc, &s2.vd};
  for (double **b : bufs)
    if (!rc) rc = alloc((void **)b, (size_t)rows * d * sizeof(double));
  if (!rc) rc = alloc((void **)&s2.flag, 16);
  ev.assign((size_t)(2 * T + 1 + 4 * (T - 1)), nullptr);
  for (cudaEvent_t &e : ev)
    if (!rc) rc = c->cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
  if (rc) {  // no helpers: the iteration stays serial
    drop_helpers();
    pipeline = 0;
  }
  return rc;
}

// Waits for and destroys the helper contexts (their own counter words restored first) and the events.
void gbk_registration::drop_helpers() {
  gbk_ctx **helpers[2] = {&c2, &c3};
  unsigned long long *words[2] = {c2_words, c3_words};
  for (int k = 0; k < 2; ++k) {
    gbk_ctx *h = *helpers[k];
    if (!h) continue;
    h->pair_counter = words[k];
    h->status = reinterpret_cast<unsigned *>(words[k] + 3);
    gbk_destroy(h);
    *helpers[k] = nullptr;
  }
  c2_words = c3_words = nullptr;
  for (cudaEvent_t e : ev)
    if (e) cudaEventDestroy(e);
  ev.clear();
}

int gbk_registration::body() {
  const long n = ncp * d;
  int rc;
  // Pipelined: the flow and the control-point adjoint run on the helper's stream, one step behind
  // the shooting and the landmark adjoint (their inputs at t and t + 1, resp. t and t - 1, are then
  // written). Serial otherwise: one stream, same launches, same results bit for bit (every launch's
  // inputs and reduction order are the same either way).
  const bool two = c2 != nullptr;
  gbk_ctx *cb = two ? c2 : c;
  const DeformScratch &sb = two ? s2 : s;
  const cudaEvent_t *ev_shoot = two ? ev.data() : nullptr, *ev_adj = two ? ev.data() + (T - 1) : nullptr;
  const cudaEvent_t ev_join0 = two ? ev[2 * T - 1] : nullptr, ev_join1 = two ? ev[2 * T] : nullptr;
  if (two) {  // the helpers launch as this context would
    for (gbk_ctx *h : {c2, c3}) {
      h->mode = c->mode;
      h->order = c->order;
      h->force_split = c->force_split;
      h->staging = c->staging;
      h->tune = c->tune;
      h->alloc_limit = c->alloc_limit;  // an injected allocation limit applies to the helpers too
      h->err.clear();
    }
  }
  // the control-point adjoint's landmark passes: beside its control-point passes on c3 when pipelined
  LandmarkSplit ls;
  ls.s = s3;
  ls.ctx = two ? c3 : nullptr;
  ls.ev = two ? ev.data() + (2 * T + 1) : nullptr;
  auto helper = [&](int r) {  // a failure of the helper chain, reported in this context
    if (r && two) c->err = c2->err;
    return r;
  };
  if ((rc = shoot_device(c, d, ncp, cp, mom, T, sigma_def, pos, momt, s, 1.0, ev_shoot, !two))) return rc;
  // regularity (reads cp and the initial momenta only: overlaps the flow): K p and
  // ConvolveGradient(cp, p) in one fused pass, <K p, p> in FP64; out = [L, L_data, L_reg, match, <Kp,p>]
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
  if ((rc = c->cuda(dot_f64(c->stream, kp, mom, n, out + 4, 0), "dot"))) return rc;
  if ((rc = c->cuda(scalar_combine(c->stream, out + 2, out + 4, -0.5, nullptr, 0, nullptr, 0), "L"))) return rc;
  c->launches += 2;
  if ((rc = helper(flow_device(cb, d, ncp, pos, momt, T, sigma_def, nv, lm0, heun, lm, sb, 1.0, ev_shoot))))
    return rc;
  if (two) {
    if ((rc = c->cuda(cudaEventRecord(ev_join0, c2->stream), "event record"))) return rc;
    if ((rc = c->cuda(cudaStreamWaitEvent(c->stream, ev_join0, 0), "event wait"))) return rc;
    if ((rc = zero_tail_device(c, d, ncp, T, momt, s))) return rc;
  }
  // data terms on the deformed template objects; thetaT = d match_k / d x_T / (2 sigma2_k)
  const double *xT = lm + (long)(T - 1) * nv * d;
  for (size_t k = 0; k < objs.size(); ++k) {
    RegObject &o = objs[k];
    if ((rc = o.surf.evaluate(c, xT + o.off * d, out + 8 + k, thetaT + o.off * d, 0.5 / o.sigma2, 0))) return rc;
  }
  if ((rc = c->cuda(gbk::launch(data_terms_kernel, 1, 1, 0, c->stream, out + 8, sigma2_dev, (int)objs.size(),
                                out + 1, out + 3),
                    "data terms")))
    return rc;
  if ((rc = c->cuda(scalar_combine(c->stream, out + 0, out + 1, 1.0, out + 2, 1.0, nullptr, 0), "L"))) return rc;
  c->launches += 2;
  if ((rc = adjoint_landmarks_device(c, d, ncp, pos, momt, T, sigma_def, nv, lm, thetaT, heun, theta, s, 1.0, nullptr,
                                     ev_adj)))
    return rc;
  if ((rc = helper(adjoint_diffeo_device(cb, d, ncp, pos, momt, T, sigma_def, nv, lm, theta, heun, xp, xm, sb, 1.0,
                                         ev_adj, &ls))))
    return rc;
  if (two) {  // (c3's passes are joined into c2's stream step by step)
    if ((rc = c->cuda(cudaEventRecord(ev_join1, c2->stream), "event record"))) return rc;
    if ((rc = c->cuda(cudaStreamWaitEvent(c->stream, ev_join1, 0), "event wait"))) return rc;
    c->launches += c2->launches + c3->launches;
    c2->launches = c3->launches = 0;
  }
  if ((rc = c->cuda(lincomb(c->stream, gmom, nullptr, -1.0, xm, -1.0, kp, n), "grad"))) return rc;
  if ((rc = c->cuda(lincomb(c->stream, gcp, nullptr, -1.0, xp, -1.0, greg, n), "grad"))) return rc;
  c->launches += 2;
  return GBK_OK;
}

int gbk_registration::run() {
  // before any capture: creates the helper contexts, buffers and events; if that fails (e.g. no device
  // memory left), the iteration runs on one stream (same results) and the message is dropped
  if (pipeline && !c2 && enable_pipeline() != GBK_OK) c->err.clear();
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

void gbk_registration::drop_graph() {
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  exec = nullptr;
  graph = nullptr;
  steps = 0;
}

void gbk_registration::release() {
  drop_graph();
  drop_helpers();
  for (RegObject &o : objs) o.surf.release();
  for (void *p : owned) cudaFree(p);
  owned.clear();
  if (stream && own_stream) cudaStreamDestroy(stream);
  stream = nullptr;
}

namespace gbk {

int registration_create(gbk_ctx *c, int d, long ncp, int nobj, const int *kinds, const long *nv_o,
                        const double *tmpl_pts, const long *nf_o, const int *cells, const long *nv_t_o,
                        const double *tgt_pts, const long *nf_t_o, const int *tgt_cells, const double *sigma_data,
                        const double *data_sigma2, int T, double sigma_def, int heun, cudaStream_t stream,
                        gbk_registration **out) {
  if (!c || !out) return GBK_ERR_ARG;
  *out = nullptr;
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "dimension %d not supported", d);
  if (nobj < 1 || !kinds || !nv_o || !nf_o || !nv_t_o || !nf_t_o || !sigma_data || !data_sigma2)
    return c->fail(GBK_ERR_ARG, "bad object description");
  if (ncp <= 0 || T < 2) return c->fail(GBK_ERR_ARG, "bad sizes");
  if (!tmpl_pts || !tgt_pts) return c->fail(GBK_ERR_ARG, "null pointer");
  // (data term kind) of each data_kind; vertices per cell follow from data_kind and d
  static const int term_kind[7] = {0, 1, 0, 1, 2, 2, 3};
  std::vector<int> cell(nobj);
  long nv = 0, nv_t = 0, ncells = 0, ncells_t = 0;
  for (int k = 0; k < nobj; ++k) {
    const int dk = kinds[k];
    if (dk < 0 || dk > 6)
      return c->fail(GBK_ERR_ARG, "data_kind must be 0/1 (surface currents/varifold), 2/3 (curve currents/varifold), "
                                  "4 (point cloud), 5 (volume mesh) or 6 (landmarks)");
    if (dk < 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "surface data terms need d = 3");
    cell[k] = dk < 2 ? 3 : dk < 4 ? 2 : dk == 5 ? d + 1 : 1;
    const long nf = cell[k] == 1 ? nv_o[k] : nf_o[k], nf_t = cell[k] == 1 ? nv_t_o[k] : nf_t_o[k];
    if (nv_o[k] <= 0 || nv_t_o[k] <= 0 || nf <= 0 || nf_t <= 0) return c->fail(GBK_ERR_ARG, "bad sizes");
    if (!(data_sigma2[k] > 0)) return c->fail(GBK_ERR_ARG, "data_sigma2 must be positive");
    if (cell[k] > 1 && (!cells || !tgt_cells)) return c->fail(GBK_ERR_ARG, "null pointer");
    nv += nv_o[k];
    nv_t += nv_t_o[k];
    if (cell[k] > 1) {
      ncells += nf * cell[k];
      ncells_t += nf_t * cell[k];
    }
  }
  gbk_registration *r = new gbk_registration();
  r->c = c;
  r->d = d;
  r->ncp = ncp;
  r->nv = nv;
  r->nv_t = nv_t;
  r->T = T;
  r->heun = heun ? 1 : 0;
  r->sigma_def = sigma_def;
  r->objs.resize(nobj);
  int rc = GBK_OK;
  if (stream) {
    r->stream = stream;
    r->own_stream = false;
  } else {
    rc = c->cuda(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking), "stream");
  }
  std::vector<int> th(ncells), tth(ncells_t);
  if (!rc && ncells) cudaMemcpy(th.data(), cells, th.size() * sizeof(int), cudaMemcpyDefault);
  if (!rc && ncells_t) cudaMemcpy(tth.data(), tgt_cells, tth.size() * sizeof(int), cudaMemcpyDefault);
  if (!rc) rc = c->cuda(cudaGetLastError(), "copy cells");
  cudaStream_t saved = c->stream;
  c->stream = r->stream;
  {
    long off = 0, co = 0, co_t = 0;
    for (int k = 0; k < nobj && !rc; ++k) {
      RegObject &o = r->objs[k];
      o.off = off;
      o.nv = nv_o[k];
      o.nv_t = nv_t_o[k];
      o.sigma2 = data_sigma2[k];
      const long nf = cell[k] == 1 ? nv_o[k] : nf_o[k], nf_t = cell[k] == 1 ? nv_t_o[k] : nf_t_o[k];
      rc = o.surf.init(c, term_kind[kinds[k]], d, cell[k], sigma_data[k], o.nv, nf, cell[k] > 1 ? th.data() + co : nullptr,
                       o.nv_t, nf_t, cell[k] > 1 ? tth.data() + co_t : nullptr);
      off += o.nv;
      if (cell[k] > 1) {
        co += nf * cell[k];
        co_t += nf_t * cell[k];
      }
    }
  }
  const long n = ncp * d, m = nv * d, rows = std::max(ncp, nv);
  struct {
    double **p;
    size_t count;
  } bufs[] = {{&r->cp, (size_t)n}, {&r->mom, (size_t)n}, {&r->pos, (size_t)T * n}, {&r->momt, (size_t)T * n},
              {&r->lm, (size_t)T * m}, {&r->lm0, (size_t)m}, {&r->theta, (size_t)T * m}, {&r->thetaT, (size_t)m},
              {&r->xp, (size_t)T * n}, {&r->xm, (size_t)T * n}, {&r->kp, (size_t)n}, {&r->greg, (size_t)n},
              {&r->gcp, (size_t)n}, {&r->gmom, (size_t)n}, {&r->out, (size_t)8 + nobj},
              {&r->sigma2_dev, (size_t)nobj}, {&r->tgt, (size_t)nv_t * d},
              {&r->s.va, (size_t)rows * d}, {&r->s.vb, (size_t)rows * d}, {&r->s.vc, (size_t)rows * d},
              {&r->s.vd, (size_t)rows * d}, {&r->s3.va, (size_t)n}, {&r->s3.vb, (size_t)n}, {&r->s3.vc, (size_t)n},
              {&r->s3.vd, (size_t)n}};
  for (auto &b : bufs)
    if (!rc) rc = r->alloc((void **)b.p, b.count * sizeof(double));
  if (!rc) rc = r->alloc((void **)&r->s.flag, 16);
  if (!rc) rc = c->cuda(cudaMemcpyAsync(r->sigma2_dev, data_sigma2, nobj * sizeof(double), cudaMemcpyHostToDevice, r->stream), "copy sigma2");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(r->tgt, tgt_pts, (size_t)nv_t * d * sizeof(double), cudaMemcpyDefault, r->stream), "copy target");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(r->lm0, tmpl_pts, (size_t)m * sizeof(double), cudaMemcpyDefault, r->stream), "copy template");
  {
    long off_t = 0;
    for (int k = 0; k < nobj && !rc; ++k) {
      gbk_ctx::OrderScope off(c, GBK_ORDER_TWO_FLOAT);
      rc = r->objs[k].surf.set_target(c, r->tgt + off_t * d);
      off_t += r->objs[k].nv_t;
    }
  }
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

}  // namespace gbk

extern "C" {

int gbk_registration_create(gbk_ctx *c, int d, long ncp, long nv, const double *tmpl_pts, long nf,
                            const int *tmpl_tris, long nv_t, const double *tgt_pts, long nf_t,
                            const int *tgt_tris, int T, double sigma_def, double sigma_data,
                            double data_sigma2, int data_kind, int heun,
                            gbk_registration **out) {
  if (!c || !out) return GBK_ERR_ARG;
  c->err.clear();
  int rc = registration_create(c, d, ncp, 1, &data_kind, &nv, tmpl_pts, &nf, tmpl_tris, &nv_t, tgt_pts, &nf_t,
                               tgt_tris, &sigma_data, &data_sigma2, T, sigma_def, heun, nullptr, out);
  if (!rc) (*out)->pipeline = pipeline_default();
  return rc;
}

int gbk_registration_create_multi(gbk_ctx *c, int d, long ncp, int nobj, const int *data_kinds, const long *nv,
                                  const double *tmpl_pts, const long *ncell, const int *tmpl_cells, const long *nv_t,
                                  const double *tgt_pts, const long *ncell_t, const int *tgt_cells,
                                  const double *sigma_data, const double *data_sigma2, int T, double sigma_def,
                                  int heun, gbk_registration **out) {
  if (!c || !out) return GBK_ERR_ARG;
  c->err.clear();
  int rc = registration_create(c, d, ncp, nobj, data_kinds, nv, tmpl_pts, ncell, tmpl_cells, nv_t, tgt_pts, ncell_t,
                               tgt_cells, sigma_data, data_sigma2, T, sigma_def, heun, nullptr, out);
  if (!rc) (*out)->pipeline = pipeline_default();
  return rc;
}

int gbk_registration_set_template(gbk_registration *r, const double *pts) {
  if (!r) return GBK_ERR_ARG;
  gbk_ctx *c = r->c;
  c->err.clear();
  GBK_RANGE();
  if (!pts) return c->fail(GBK_ERR_ARG, "null pointer");
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  int rc = c->cuda(cudaMemcpyAsync(r->lm0, pts, (size_t)r->nv * r->d * sizeof(double), cudaMemcpyDefault, r->stream),
                   "copy template");
  if (!rc) rc = c->cuda(cudaStreamSynchronize(r->stream), "sync");
  return rc;
}

int gbk_registration_set_point_weights(gbk_registration *r, const double *w_tmpl, const double *w_tgt) {
  if (!r) return GBK_ERR_ARG;
  gbk_ctx *c = r->c;
  c->err.clear();
  GBK_RANGE();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  cudaStream_t saved = c->stream;
  c->stream = r->stream;
  int rc = GBK_OK, clouds = 0;
  {
    gbk_ctx::OrderScope off(c, GBK_ORDER_TWO_FLOAT);
    long off_t = 0;
    for (RegObject &o : r->objs) {
      if (o.surf.kind == 2 && o.surf.cell == 1) {  // same buffers: a captured graph reads the new weights
        ++clouds;
        if (!rc) rc = o.surf.set_weights(c, w_tmpl ? w_tmpl + o.off : nullptr, w_tgt ? w_tgt + off_t : nullptr);
      }
      off_t += o.nv_t;
    }
  }
  c->stream = saved;
  if (!rc && !clouds) rc = c->fail(GBK_ERR_STATE, "the registration has no point-cloud object");
  return rc;
}

int gbk_registration_set_graph(gbk_registration *r, int enable) {
  if (!r) return GBK_ERR_ARG;
  r->use_graph = enable ? 1 : 0;
  return GBK_OK;
}

int gbk_registration_step(gbk_registration *r, const double *cp, const double *mom, double *loglik,
                          double *grad_cp, double *grad_mom) {
  if (!r) return GBK_ERR_ARG;
  gbk_ctx *c = r->c;
  c->err.clear();
  GBK_RANGE();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (!cp || !mom) return c->fail(GBK_ERR_ARG, "null pointer");
  const size_t nb = (size_t)r->ncp * r->d * sizeof(double);
  int rc = c->cuda(cudaMemcpyAsync(r->cp, cp, nb, cudaMemcpyDefault, r->stream), "copy cp");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(r->mom, mom, nb, cudaMemcpyDefault, r->stream), "copy mom");
  if (!rc) {
    gbk_ctx::OrderScope off(c, GBK_ORDER_TWO_FLOAT);
    rc = r->run();
  }
  if (!rc && loglik) rc = c->cuda(cudaMemcpyAsync(loglik, r->out, 5 * sizeof(double), cudaMemcpyDefault, r->stream), "copy L");
  if (!rc && grad_cp) rc = c->cuda(cudaMemcpyAsync(grad_cp, r->gcp, nb, cudaMemcpyDefault, r->stream), "copy grad");
  if (!rc && grad_mom) rc = c->cuda(cudaMemcpyAsync(grad_mom, r->gmom, nb, cudaMemcpyDefault, r->stream), "copy grad");
  if (!rc) rc = c->cuda(cudaStreamSynchronize(r->stream), "sync");
  return rc;
}

int gbk_registration_trajectories(gbk_registration *r, double *pos, double *mom, double *lm,
                                  double *theta, double *xi_pos, double *xi_mom) {
  if (!r) return GBK_ERR_ARG;
  gbk_ctx *c = r->c;
  const size_t n = (size_t)r->T * r->ncp * r->d * sizeof(double), m = (size_t)r->T * r->nv * r->d * sizeof(double);
  int rc = GBK_OK;
  auto cp = [&](double *dst, const double *src, size_t bytes) {
    if (!rc && dst) rc = c->cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, r->stream), "copy");
  };
  cp(pos, r->pos, n);
  cp(mom, r->momt, n);
  cp(lm, r->lm, m);
  cp(theta, r->theta, m);
  cp(xi_pos, r->xp, n);
  cp(xi_mom, r->xm, n);
  if (!rc) rc = c->cuda(cudaStreamSynchronize(r->stream), "sync");
  return rc;
}

long long gbk_registration_graph_launches(const gbk_registration *r) { return r ? r->graph_launches : 0; }

// Nesterov-accelerated gradient ascent of the registration log-likelihood over the control points
// and momenta (FastGradientAscent.cxx:48-300, gbk_optimize.cu): every parameter, trial point and
// gradient stays on the device; each evaluation is one replay of the iteration graph and one
// 40-byte read of the log-likelihood terms (plus the squared gradient norms after an accepted
// step) for the line-search decisions, which the host takes.
int gbk_registration_optimize(gbk_registration *r, double *cp, double *mom, int optimize_cp, int max_iterations,
                              double initial_step, int max_line_search, double shrink, double expand,
                              double tolerance, int nb_iter_freeze, double *history, int *iterations,
                              double *info, double *aux_cp, double *aux_mom, double *grad_cp,
                              double *grad_mom) {
  if (!r) return GBK_ERR_ARG;
  gbk_ctx *c = r->c;
  c->err.clear();
  GBK_RANGE();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (!cp || !mom || !history || !iterations) return c->fail(GBK_ERR_ARG, "null pointer");
  const long n = r->ncp * r->d;
  const size_t nb = (size_t)n * sizeof(double);
  gbk_ctx::OrderScope off(c, GBK_ORDER_TWO_FLOAT);
  cudaStream_t st = r->stream;
  double *sq_dev = nullptr;
  int rc = c->cuda(cudaMalloc(&sq_dev, 4 * sizeof(double)), "cudaMalloc (optimiser)");
  if (!rc && !optimize_cp) rc = c->cuda(cudaMemcpyAsync(r->cp, cp, nb, cudaMemcpyDefault, st), "copy cp");
  // groups: [control points,] momenta
  const int ng = optimize_cp ? 2 : 1;
  const long sizes[2] = {n, n};
  double *params[2] = {optimize_cp ? cp : mom, mom};
  double *aux_out[2] = {optimize_cp ? aux_cp : aux_mom, aux_mom};
  double *grad_out[2] = {optimize_cp ? grad_cp : grad_mom, grad_mom};
  FgaEvaluate ev = [&](double *const *p, bool need_grad, double *terms, double *const *g, double *sq) -> int {
    int e = GBK_OK;
    if (optimize_cp) e = c->cuda(cudaMemcpyAsync(r->cp, p[0], nb, cudaMemcpyDeviceToDevice, st), "copy cp");
    if (!e) e = c->cuda(cudaMemcpyAsync(r->mom, p[ng - 1], nb, cudaMemcpyDeviceToDevice, st), "copy mom");
    if (!e) e = r->run();
    double out[5];
    if (!e) e = c->cuda(cudaMemcpyAsync(out, r->out, sizeof out, cudaMemcpyDeviceToHost, st), "read L");
    double h[2] = {0, 0};
    if (!e && need_grad) {
      if (optimize_cp) e = c->cuda(cudaMemcpyAsync(g[0], r->gcp, nb, cudaMemcpyDeviceToDevice, st), "copy grad");
      if (!e) e = c->cuda(cudaMemcpyAsync(g[ng - 1], r->gmom, nb, cudaMemcpyDeviceToDevice, st), "copy grad");
      if (!e) e = c->cuda(dot_f64(st, r->gcp, r->gcp, n, sq_dev, 0), "grad norm");
      if (!e) e = c->cuda(dot_f64(st, r->gmom, r->gmom, n, sq_dev + 1, 0), "grad norm");
      if (!e) e = c->cuda(cudaMemcpyAsync(h, sq_dev, sizeof h, cudaMemcpyDeviceToHost, st), "read norms");
    }
    if (!e) e = c->cuda(cudaStreamSynchronize(st), "sync");
    if (!e) {
      terms[0] = out[1];
      terms[1] = out[2];
      if (need_grad) {
        if (optimize_cp) sq[0] = h[0];
        sq[ng - 1] = h[1];
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
  if (!rc) rc = fast_gradient_ascent(c, st, ng, sizes, params, o, ev, &res, aux_out, grad_out);
  if (sq_dev) cudaFree(sq_dev);
  if (rc) return rc;
  std::copy(res.history.begin(), res.history.end(), history);
  *iterations = res.rows;
  if (info) {
    info[0] = res.step[0];
    info[1] = res.step[ng - 1];
    info[2] = res.tau;
    info[3] = res.freeze;
    info[4] = res.sq[0];
    info[5] = res.sq[ng - 1];
    info[6] = (double)res.evaluations;
    info[7] = res.stop;
  }
  return GBK_OK;
}

void gbk_registration_destroy(gbk_registration *r) {
  if (!r) return;
  cudaSetDevice(r->c->device);
  if (r->stream) cudaStreamSynchronize(r->stream);
  r->release();
  delete r;
}

}  // extern "C"
