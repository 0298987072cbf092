// One registration iteration of a subject of DeterministicAtlas with a frozen template, on the
// device, replayed from a CUDA graph.
//
// Log-likelihood (DeterministicAtlas.cxx:99-154) L = -0.5 match / data_sigma2 - 0.5 <K p, p>
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
#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_deform_impl.h"
#include "gbk_dispatch.h"
#include "gbk_geometry.h"
#include "gbk_hostio.h"
#include "gbk_ops.h"

using namespace gbk;

struct gbk_registration {
  gbk_ctx *c = nullptr;
  int d = 3, T = 2, heun = 1, use_graph = 1, steps = 0;
  long ncp = 0, nv = 0;
  double sigma_def = 1, sigma_data = 1, data_sigma2 = 1;
  cudaStream_t stream = nullptr;
  SurfaceTerm surf;
  std::vector<void *> owned;
  double *cp = nullptr, *mom = nullptr, *pos = nullptr, *momt = nullptr, *lm = nullptr, *lm0 = nullptr;
  double *theta = nullptr, *thetaT = nullptr, *xp = nullptr, *xm = nullptr;
  double *kp = nullptr, *greg = nullptr, *gcp = nullptr, *gmom = nullptr, *out = nullptr;
  DeformScratch s;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;

  int alloc(void **p, size_t bytes) {
    cudaError_t e = cudaMalloc(p, std::max(bytes, (size_t)8));
    if (e != cudaSuccess) return c->cuda(e, "cudaMalloc (registration)");
    owned.push_back(*p);
    return GBK_OK;
  }

  // The whole iteration on `stream`, device pointers only.
  int body() {
    const long n = ncp * d;
    int rc;
    if ((rc = shoot_device(c, d, ncp, cp, mom, T, sigma_def, pos, momt, s))) return rc;
    if ((rc = flow_device(c, d, ncp, pos, momt, T, sigma_def, nv, lm0, heun, lm, s))) return rc;
    // data term on the deformed template; thetaT = d match / d x_T / (2 data_sigma2)
    if ((rc = surf.evaluate(c, lm + (long)(T - 1) * nv * d, out + 3, thetaT, 0.5 / data_sigma2, 0))) return rc;
    // regularity: K p and ConvolveGradient(cp, p) in one fused pass, <K p, p> in FP64
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
    // out = [L, L_data, L_reg, match, <Kp,p>]
    if ((rc = c->cuda(scalar_combine(c->stream, out + 1, out + 3, -0.5 / data_sigma2, nullptr, 0, nullptr, 0), "L"))) return rc;
    if ((rc = c->cuda(scalar_combine(c->stream, out + 2, out + 4, -0.5, nullptr, 0, nullptr, 0), "L"))) return rc;
    if ((rc = c->cuda(scalar_combine(c->stream, out + 0, out + 1, 1.0, out + 2, 1.0, nullptr, 0), "L"))) return rc;
    c->launches += 4;
    if ((rc = adjoint_landmarks_device(c, d, ncp, pos, momt, T, sigma_def, nv, lm, thetaT, heun, theta, s))) return rc;
    if ((rc = adjoint_diffeo_device(c, d, ncp, pos, momt, T, sigma_def, nv, lm, theta, heun, xp, xm, s))) return rc;
    if ((rc = c->cuda(lincomb(c->stream, gmom, nullptr, -1.0, xm, -1.0, kp, n), "grad"))) return rc;
    if ((rc = c->cuda(lincomb(c->stream, gcp, nullptr, -1.0, xp, -1.0, greg, n), "grad"))) return rc;
    c->launches += 2;
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
  long long graph_launches = 0;

  void release() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
    surf.release();
    for (void *p : owned) cudaFree(p);
    owned.clear();
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
  }
};

extern "C" {

int gbk_registration_create(gbk_ctx *c, int d, long ncp, long nv, const double *tmpl_pts, long nf,
                            const int *tmpl_tris, long nv_t, const double *tgt_pts, long nf_t,
                            const int *tgt_tris, int T, double sigma_def, double sigma_data,
                            double data_sigma2, int data_kind, int heun,
                            gbk_registration **out) {
  if (!c || !out) return GBK_ERR_ARG;
  *out = nullptr;
  c->err.clear();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "surface registration needs d = 3");
  if (ncp <= 0 || nv <= 0 || nf <= 0 || nv_t <= 0 || nf_t <= 0 || T < 2)
    return c->fail(GBK_ERR_ARG, "bad sizes");
  if (data_kind != 0 && data_kind != 1) return c->fail(GBK_ERR_ARG, "data_kind must be 0 (currents) or 1 (varifold)");
  if (!(data_sigma2 > 0)) return c->fail(GBK_ERR_ARG, "data_sigma2 must be positive");
  if (!tmpl_pts || !tmpl_tris || !tgt_pts || !tgt_tris) return c->fail(GBK_ERR_ARG, "null pointer");
  gbk_registration *r = new gbk_registration();
  r->c = c;
  r->d = d;
  r->ncp = ncp;
  r->nv = nv;
  r->T = T;
  r->heun = heun ? 1 : 0;
  r->sigma_def = sigma_def;
  r->sigma_data = sigma_data;
  r->data_sigma2 = data_sigma2;
  int rc = c->cuda(cudaStreamCreateWithFlags(&r->stream, cudaStreamNonBlocking), "stream");
  std::vector<int> th((size_t)nf * 3), tth((size_t)nf_t * 3);
  if (!rc) {
    cudaMemcpy(th.data(), tmpl_tris, th.size() * sizeof(int), cudaMemcpyDefault);
    cudaMemcpy(tth.data(), tgt_tris, tth.size() * sizeof(int), cudaMemcpyDefault);
    rc = c->cuda(cudaGetLastError(), "copy triangles");
  }
  cudaStream_t saved = c->stream;
  c->stream = r->stream;
  if (!rc) rc = r->surf.init(c, data_kind, sigma_data, nv, nf, th.data(), nv_t, nf_t, tth.data());
  const long n = ncp * d, m = nv * d, rows = std::max(ncp, nv);
  struct {
    double **p;
    size_t count;
  } bufs[] = {{&r->cp, (size_t)n}, {&r->mom, (size_t)n}, {&r->pos, (size_t)T * n}, {&r->momt, (size_t)T * n},
              {&r->lm, (size_t)T * m}, {&r->lm0, (size_t)m}, {&r->theta, (size_t)T * m}, {&r->thetaT, (size_t)m},
              {&r->xp, (size_t)T * n}, {&r->xm, (size_t)T * n}, {&r->kp, (size_t)n}, {&r->greg, (size_t)n},
              {&r->gcp, (size_t)n}, {&r->gmom, (size_t)n}, {&r->out, 8},
              {&r->s.va, (size_t)rows * d}, {&r->s.vb, (size_t)rows * d}, {&r->s.vc, (size_t)rows * d},
              {&r->s.vd, (size_t)rows * d}};
  for (auto &b : bufs)
    if (!rc) rc = r->alloc((void **)b.p, b.count * sizeof(double));
  if (!rc) rc = r->alloc((void **)&r->s.flag, 16);
  double *tgt_dev = nullptr;
  if (!rc) rc = r->alloc((void **)&tgt_dev, (size_t)nv_t * 3 * sizeof(double));
  if (!rc) rc = c->cuda(cudaMemcpyAsync(tgt_dev, tgt_pts, (size_t)nv_t * 3 * sizeof(double), cudaMemcpyDefault, r->stream), "copy target");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(r->lm0, tmpl_pts, (size_t)m * sizeof(double), cudaMemcpyDefault, r->stream), "copy template");
  if (!rc) rc = r->surf.set_target(c, tgt_dev);
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
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (!cp || !mom) return c->fail(GBK_ERR_ARG, "null pointer");
  const size_t nb = (size_t)r->ncp * r->d * sizeof(double);
  int rc = c->cuda(cudaMemcpyAsync(r->cp, cp, nb, cudaMemcpyDefault, r->stream), "copy cp");
  if (!rc) rc = c->cuda(cudaMemcpyAsync(r->mom, mom, nb, cudaMemcpyDefault, r->stream), "copy mom");
  if (!rc) {
    gbk_ctx::OrderScope off(c, GBK_ORDER_OFF);
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

void gbk_registration_destroy(gbk_registration *r) {
  if (!r) return;
  cudaSetDevice(r->c->device);
  if (r->stream) cudaStreamSynchronize(r->stream);
  r->release();
  delete r;
}

}  // extern "C"
