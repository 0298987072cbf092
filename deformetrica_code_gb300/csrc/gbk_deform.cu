// Device-resident geodesic shooting, landmark flow and adjoint integration.
//
// Each loop of the reference runs here as a sequence of fused pair passes plus small FP64
// element-wise kernels on one stream, with no host synchronisation inside the loop:
//   Diffeos::Shoot (Diffeos.cxx:589-660): per step ONE pass of the fused Convolve + alpha-gradient
//     op over CP x CP (dPos = K p and dMom = G^T p, the reference's varlin call + host contraction
//     at :624-630), then the Euler update;
//   Diffeos::FlowLandmarkPointsTrajectory (:661-712): Convolve V x CP per stage, Heun optional;
//   IntegrateAdjointOfLandmarkPointsEquations (AdjointEquationsIntegrator.cxx:59-136): the
//     alpha-gradient V x CP per stage;
//   ComputeUpdateAt (:476-570): ONE fused CP x CP pass (OpAdjointCP, replacing five kernel calls)
//     plus ONE fused CP x V pass (Convolve + alpha-gradient of the landmark adjoint, :519-521);
//   IntegrateAdjointOfDiffeoParametersEquations (:414-470): Euler / Heun over ComputeUpdateAt.
// Trajectories are T x n x d row-major blocks. The reference's "nearly zero momenta" shortcuts
// (Diffeos.cxx:611-613, :683-684) are taken on the device through a flag, so results match them
// exactly without a host round trip.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_deform_impl.h"
#include "gbk_dispatch.h"
#include "gbk_hostio.h"
#include "gbk_ops.h"

namespace gbk {

// ---------------------------------------------------------------------------------------------
// element-wise and reduction kernels
// ---------------------------------------------------------------------------------------------
__global__ void lincomb_kernel(double *out, const double *base, double c1, const double *v1,
                               double c2, const double *v2, long n, const int *flag,
                               const double *flag_value) {
  pdl_entry();
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (flag && *flag) {
    out[i] = flag_value ? flag_value[i] : (base ? base[i] : 0.0);
    return;
  }
  double r = base ? base[i] : 0.0;
  if (v1) r += c1 * v1[i];
  if (v2) r += c2 * v2[i];
  out[i] = r;
}

__global__ void __launch_bounds__(1024) norm_flag_kernel(const double *p, long n, double thresh,
                                                         int *flag) {
  pdl_entry();
  __shared__ double s[1024];
  double acc = 0.0;
  for (long i = threadIdx.x; i < n; i += blockDim.x) acc = fma(p[i], p[i], acc);
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *flag = sqrt(s[0]) < thresh ? 1 : 0;
}

__global__ void __launch_bounds__(1024) dot_kernel(const double *a, const double *b, long n,
                                                   double *out, int accumulate) {
  pdl_entry();
  __shared__ double s[1024];
  double acc = 0.0;
  for (long i = threadIdx.x; i < n; i += blockDim.x) acc = fma(a[i], b[i], acc);
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = accumulate ? *out + s[0] : s[0];
}

__global__ void scalar_combine_kernel(double *out, const double *a, double alpha, const double *b,
                                      double beta, const double *c, double gamma) {
  pdl_entry();
  double r = 0.0;
  if (a) r += alpha * *a;
  if (b) r += beta * *b;
  if (c) r += gamma * *c;
  *out = r;
}

__global__ void zero_if_flag_kernel(double *p, long n, const int *flag) {
  pdl_entry();
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && *flag) p[i] = 0.0;
}

// out = base + c1 v1 + c2 v2 + c3 v3 + c4 v4, added in that order (the Heun corrector of the
// control-point adjoint with its landmark terms kept apart)
__global__ void lincomb4_kernel(double *out, const double *base, double c1, const double *v1, double c2,
                                const double *v2, double c3, const double *v3, double c4, const double *v4, long n) {
  pdl_entry();
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double r = base[i];
  r += c1 * v1[i];
  r += c2 * v2[i];
  r += c3 * v3[i];
  r += c4 * v4[i];
  out[i] = r;
}

static unsigned blocks_for(long n, int bs = 256) { return (unsigned)std::max(1L, (n + bs - 1) / bs); }

cudaError_t lincomb(cudaStream_t st, double *out, const double *base, double c1, const double *v1,
                    double c2, const double *v2, long n, const int *flag, const double *flag_value) {
  if (n <= 0) return cudaSuccess;
  return launch(lincomb_kernel, blocks_for(n), 256, 0, st, out, base, c1, v1, c2, v2, n, flag, flag_value);
}

cudaError_t small_norm_flag(cudaStream_t st, const double *p, long n, double thresh, int *flag) {
  return launch(norm_flag_kernel, 1, 1024, 0, st, p, n, thresh, flag);
}

cudaError_t dot_f64(cudaStream_t st, const double *a, const double *b, long n, double *out,
                    int accumulate) {
  return launch(dot_kernel, 1, 1024, 0, st, a, b, n, out, accumulate);
}

cudaError_t scalar_combine(cudaStream_t st, double *out, const double *a, double alpha,
                           const double *b, double beta, const double *c, double gamma) {
  return launch(scalar_combine_kernel, 1, 1, 0, st, out, a, alpha, b, beta, c, gamma);
}

// ---------------------------------------------------------------------------------------------
// loop bodies (device pointers only; shared with the registration object)
// ---------------------------------------------------------------------------------------------
int shoot_device(gbk_ctx *c, int d, long ncp, const double *cp0, const double *mom0, int T,
                 double sigma, double *pos, double *mom, const DeformScratch &s, double span,
                 const cudaEvent_t *step_done, bool zero_tail) {
  const long n = ncp * d;
  const double dt = span / (T - 1);
  cudaStream_t st = c->stream;
  int rc;
  if ((rc = c->cuda(cudaMemcpyAsync(pos, cp0, n * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy")))
    return rc;
  if ((rc = c->cuda(cudaMemcpyAsync(mom, mom0, n * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy")))
    return rc;
  if ((rc = c->cuda(small_norm_flag(st, mom0, n, 1e-20, s.flag), "norm flag"))) return rc;
  c->launches += 1;
  for (int t = 0; t + 1 < T; ++t) {
    const double *pt = pos + t * n, *mt = mom + t * n;
    PairArgs a = pair_args(ncp, ncp, sigma);
    a.x = pt;
    a.y = pt;
    a.w = mt;
    a.w_ld = d;
    a.ta = mt;
    a.ta_ld = d;
    // dPos = K p, dMom = G^T p, and the explicit Euler step fused into the stores:
    // pos[t+1] = pos[t] + dt dPos ; mom[t+1] = mom[t] - dt dMom (Diffeos.cxx:631-632); with nearly zero
    // momenta pos stays cp0 and mom[t+1] = mom[t] (zeroed below) (:601-613)
    a.out0 = pos + (t + 1) * n;
    a.out0_ld = d;
    a.base0 = pt;
    a.step0 = dt;
    a.flag_out0 = cp0;
    a.out1 = mom + (t + 1) * n;
    a.out1_ld = d;
    a.base1 = mt;
    a.step1 = -dt;
    a.flag = s.flag;
    if ((rc = c->launch(OP_CONV_GRADA, d, d, a))) return rc;
    if (step_done && (rc = c->cuda(cudaEventRecord(step_done[t], st), "event record"))) return rc;
  }
  return zero_tail ? zero_tail_device(c, d, ncp, T, mom, s) : GBK_OK;
}

// nearly zero momenta: the reference leaves mom[t >= 1] at their initial zeros (Diffeos.cxx:601-613)
int zero_tail_device(gbk_ctx *c, int d, long ncp, int T, double *mom, const DeformScratch &s) {
  const long n = ncp * d;
  c->launches += 1;
  return c->cuda(launch(zero_if_flag_kernel, blocks_for((T - 1) * n), 256, 0, c->stream, mom + n, (T - 1) * n,
                        s.flag),
                 "zero_if_flag_kernel");
}

int flow_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom, int T,
                double sigma, long nlm, const double *lm0, int heun, double *lm,
                const DeformScratch &s, double span, const cudaEvent_t *wait_step) {
  const long n = ncp * d, m = nlm * d;
  const double dt = span / (T - 1);
  cudaStream_t st = c->stream;
  int rc;
  if (wait_step && (rc = c->cuda(cudaStreamWaitEvent(st, wait_step[0], 0), "event wait"))) return rc;
  if ((rc = c->cuda(cudaMemcpyAsync(lm, lm0, m * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy"))) return rc;
  if ((rc = c->cuda(small_norm_flag(st, mom, n, 1e-20, s.flag), "norm flag"))) return rc;
  c->launches += 1;
  for (int t = 0; t + 1 < T; ++t) {
    if (wait_step && t > 0 && (rc = c->cuda(cudaStreamWaitEvent(st, wait_step[t], 0), "event wait"))) return rc;
    const double *lt = lm + t * m;
    double *lt1 = lm + (t + 1) * m;
    PairArgs a = pair_args(nlm, ncp, sigma);
    a.x = lt;
    a.y = pos + t * n;
    a.w = mom + t * n;
    a.w_ld = d;
    a.out0 = s.vc;
    a.out0_ld = d;
    if ((rc = c->launch(OP_CONV, d, d, a))) return rc;
    if ((rc = c->cuda(lincomb(st, lt1, lt, dt, s.vc, 0, nullptr, m, s.flag, nullptr), "euler"))) return rc;
    c->launches += 1;
    if (heun) {  // the Heun corrector fused into the store: lt1 = lt + dt/2 vc + dt/2 K(lt1) p (in place)
      PairArgs b = pair_args(nlm, ncp, sigma);
      b.x = lt1;
      b.y = pos + (t + 1) * n;
      b.w = mom + (t + 1) * n;
      b.w_ld = d;
      b.out0 = lt1;
      b.out0_ld = d;
      b.base0 = lt;
      b.aux0 = s.vc;
      b.aux_c0 = 0.5 * dt;
      b.step0 = 0.5 * dt;
      b.flag = s.flag;
      if ((rc = c->launch(OP_CONV, d, d, b))) return rc;
    }
  }
  return GBK_OK;
}

int adjoint_landmarks_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom,
                             int T, double sigma, long nlm, const double *lm,
                             const double *theta_final, int heun, double *theta,
                             const DeformScratch &s, double span, const AdjointJumps *jumps,
                             const cudaEvent_t *step_done) {
  const long n = ncp * d, m = nlm * d;
  const double dt = span / (T - 1);
  cudaStream_t st = c->stream;
  int rc;
  // observations: the reference's jumps (several observations), or each gradient added at its own
  // time index; one reference observation is the plain final condition
  const bool obs = jumps && jumps->n > 0;
  const bool ref_jumps = obs && jumps->reference && jumps->n > 1;
  const bool own_index = obs && !jumps->reference;
  int si = obs ? jumps->n - 1 : 0;
  double *thT = theta + (T - 1) * m;
  if (obs && jumps->reference && jumps->n == 1) {
    rc = c->cuda(cudaMemcpyAsync(thT, jumps->grads[0], m * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
  } else if (ref_jumps && jumps->times[si] == T - 1) {
    rc = c->cuda(cudaMemcpyAsync(thT, jumps->grads[si], m * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
    si = si > 0 ? si - 1 : 0;
  } else if (obs) {
    rc = c->cuda(lincomb(st, thT, nullptr, 0.0, nullptr, 0.0, nullptr, m), "zero");
    c->launches += 1;
    for (int k = 0; k < jumps->n && !rc && own_index; ++k)
      if (jumps->times[k] == T - 1) {
        rc = c->cuda(lincomb(st, thT, thT, 1.0, jumps->grads[k], 0.0, nullptr, m), "jump");
        c->launches += 1;
      }
  } else {
    rc = c->cuda(cudaMemcpyAsync(thT, theta_final, m * sizeof(double), cudaMemcpyDeviceToDevice, st), "copy");
  }
  if (rc) return rc;
  for (int t = T - 1; t > 0; --t) {
    PairArgs a = pair_args(nlm, ncp, sigma);
    a.x = lm + t * m;
    a.ta = theta + t * m;
    a.ta_ld = d;
    a.y = pos + t * n;
    a.w = mom + t * n;
    a.w_ld = d;
    a.out1 = s.vc;
    a.out1_ld = d;
    if ((rc = c->launch(OP_GRADA, d, d, a))) return rc;
    // the reference adds the observation's gradient to the rate (AdjointEquationsIntegrator.cxx:104-109)
    const bool jump_here = ref_jumps && t == jumps->times[si];
    if (jump_here) {
      if ((rc = c->cuda(lincomb(st, s.vc, s.vc, 1.0, jumps->grads[si], 0.0, nullptr, m), "jump"))) return rc;
      c->launches += 1;
    }
    double *th1 = theta + (t - 1) * m;
    if ((rc = c->cuda(lincomb(st, th1, theta + t * m, dt, s.vc, 0, nullptr, m), "euler"))) return rc;
    c->launches += 1;
    if (heun) {
      PairArgs b = pair_args(nlm, ncp, sigma);
      b.x = lm + (t - 1) * m;
      b.ta = th1;
      b.ta_ld = d;
      b.y = pos + (t - 1) * n;
      b.w = mom + (t - 1) * n;
      b.w_ld = d;
      if (!jump_here) {  // the Heun corrector fused into the store: th1 = th_t + dt/2 vc + dt/2 vd (in place)
        b.out1 = th1;
        b.out1_ld = d;
        b.base1 = theta + t * m;
        b.aux1 = s.vc;
        b.aux_c1 = 0.5 * dt;
        b.step1 = 0.5 * dt;
        if ((rc = c->launch(OP_GRADA, d, d, b))) return rc;
      } else {
        b.out1 = s.vd;
        b.out1_ld = d;
        if ((rc = c->launch(OP_GRADA, d, d, b))) return rc;
        // and the cursor moves back in this branch only (:123-128)
        if ((rc = c->cuda(lincomb(st, s.vd, s.vd, 1.0, jumps->grads[si], 0.0, nullptr, m), "jump"))) return rc;
        c->launches += 1;
        si = si > 0 ? si - 1 : 0;
        if ((rc = c->cuda(lincomb(st, th1, theta + t * m, 0.5 * dt, s.vc, 0.5 * dt, s.vd, m), "heun"))) return rc;
        c->launches += 1;
      }
    }
    for (int k = 0; k < (own_index ? jumps->n : 0); ++k)
      if (jumps->times[k] == t - 1) {
        if ((rc = c->cuda(lincomb(st, th1, th1, 1.0, jumps->grads[k], 0.0, nullptr, m), "jump"))) return rc;
        c->launches += 1;
      }
    if (step_done && (rc = c->cuda(cudaEventRecord(step_done[t], st), "event record"))) return rc;
  }
  return GBK_OK;
}

// The control-point pass of ComputeUpdateAt (OpAdjointCP: dXi3 .. dXi6), written to dpos / dmom.
static int update_cp_pass(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom, const double *xp,
                          const double *xm, double sigma, double *dpos, double *dmom) {
  PairArgs a = pair_args(ncp, ncp, sigma);
  a.x = pos;
  a.y = pos;
  a.ta = mom;
  a.ta_ld = d;
  a.w = mom;
  a.w_ld = d;
  a.tb = xp;
  a.tb_ld = d;
  a.sb = xm;
  a.sb_ld = d;
  a.out0 = dpos;
  a.out0_ld = d;
  a.out1 = dmom;
  a.out1_ld = d;
  return c->launch(OP_ADJCP, d, d, a);
}

// The landmark pass of ComputeUpdateAt: dXi1 = ConvolveGradient(pos, mom) and dXi2 = Convolve(pos)
// with sources lm, weights theta (AdjointEquationsIntegrator.cxx:519-521), one fused pass, written
// to (acc = 0) or added into (acc = 1) dpos / dmom.
static int update_landmark_pass(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom, long nlm,
                                const double *lm, const double *theta, double sigma, double *dpos, double *dmom,
                                int acc) {
  PairArgs b = pair_args(ncp, nlm, sigma);
  b.x = pos;
  b.ta = mom;
  b.ta_ld = d;
  b.y = lm;
  b.w = theta;
  b.w_ld = d;
  b.out0 = dmom;
  b.out0_ld = d;
  b.acc0 = acc;
  b.out1 = dpos;
  b.out1_ld = d;
  b.acc1 = acc;
  return c->launch(OP_CONV_GRADA, d, d, b);
}

int update_at_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom,
                     const double *xp, const double *xm, long nlm, const double *lm,
                     const double *theta, double sigma, double *dpos, double *dmom) {
  int rc = update_cp_pass(c, d, ncp, pos, mom, xp, xm, sigma, dpos, dmom);
  if (rc || nlm <= 0) return rc;
  return update_landmark_pass(c, d, ncp, pos, mom, nlm, lm, theta, sigma, dpos, dmom, 1);
}

int adjoint_diffeo_device(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom, int T,
                          double sigma, long nlm, const double *lm, const double *theta, int heun,
                          double *xp, double *xm, const DeformScratch &s, double span,
                          const cudaEvent_t *wait_step, const LandmarkSplit *split) {
  const long n = ncp * d, m = nlm * d;
  const double dt = span / (T - 1);
  cudaStream_t st = c->stream;
  int rc;
  const LandmarkSplit *ls = nlm > 0 ? split : nullptr;
  // ComputeUpdateAt at time index k into (dpos, dmom); with a split, its landmark terms go to
  // (lpos, lmom) instead, on the split's context (concurrently, between fork / join events e, e + 1)
  // or on this one
  auto update = [&](long k, const double *xpk, const double *xmk, double *dpos, double *dmom, double *lpos,
                    double *lmom, int e) -> int {
    const double *lmk = nlm ? lm + k * m : nullptr, *thk = nlm ? theta + k * m : nullptr;
    if (!ls) return update_at_device(c, d, ncp, pos + k * n, mom + k * n, xpk, xmk, nlm, lmk, thk, sigma, dpos, dmom);
    gbk_ctx *cl = ls->ctx ? ls->ctx : c;
    int r;
    if (ls->ctx) {
      if ((r = c->cuda(cudaEventRecord(ls->ev[e], st), "event record"))) return r;
      if ((r = c->cuda(cudaStreamWaitEvent(cl->stream, ls->ev[e], 0), "event wait"))) return r;
    }
    if ((r = update_landmark_pass(cl, d, ncp, pos + k * n, mom + k * n, nlm, lmk, thk, sigma, lpos, lmom, 0))) {
      if (cl != c) c->err = cl->err;
      return r;
    }
    if (ls->ctx && (r = c->cuda(cudaEventRecord(ls->ev[e + 1], cl->stream), "event record"))) return r;
    if ((r = update_cp_pass(c, d, ncp, pos + k * n, mom + k * n, xpk, xmk, sigma, dpos, dmom))) return r;
    if (ls->ctx && (r = c->cuda(cudaStreamWaitEvent(st, ls->ev[e + 1], 0), "event wait"))) return r;
    return GBK_OK;
  };
  if (wait_step && (rc = c->cuda(cudaStreamWaitEvent(st, wait_step[T - 1], 0), "event wait"))) return rc;
  if ((rc = c->cuda(cudaMemsetAsync(xp + (T - 1) * n, 0, n * sizeof(double), st), "memset"))) return rc;
  if ((rc = c->cuda(cudaMemsetAsync(xm + (T - 1) * n, 0, n * sizeof(double), st), "memset"))) return rc;
  for (int t = T - 1; t > 0; --t) {
    if (wait_step && t < T - 1 && (rc = c->cuda(cudaStreamWaitEvent(st, wait_step[t], 0), "event wait"))) return rc;
    const int e = 4 * (T - 1 - t);
    if ((rc = update(t, xp + t * n, xm + t * n, s.va, s.vb, ls ? ls->s.va : nullptr, ls ? ls->s.vb : nullptr, e)))
      return rc;
    double *xp1 = xp + (t - 1) * n, *xm1 = xm + (t - 1) * n;
    if ((rc = c->cuda(lincomb(st, xp1, xp + t * n, dt, s.va, ls ? dt : 0, ls ? ls->s.va : nullptr, n), "euler")))
      return rc;
    if ((rc = c->cuda(lincomb(st, xm1, xm + t * n, dt, s.vb, ls ? dt : 0, ls ? ls->s.vb : nullptr, n), "euler")))
      return rc;
    c->launches += 2;
    if (heun) {
      if ((rc = update(t - 1, xp1, xm1, s.vc, s.vd, ls ? ls->s.vc : nullptr, ls ? ls->s.vd : nullptr, e + 2)))
        return rc;
      if (ls) {
        const double h = 0.5 * dt;
        if ((rc = c->cuda(launch(lincomb4_kernel, blocks_for(n), 256, 0, st, xp1, xp + t * n, h, s.va, h, ls->s.va, h,
                                 s.vc, h, ls->s.vc, n),
                          "heun")))
          return rc;
        if ((rc = c->cuda(launch(lincomb4_kernel, blocks_for(n), 256, 0, st, xm1, xm + t * n, h, s.vb, h, ls->s.vb, h,
                                 s.vd, h, ls->s.vd, n),
                          "heun")))
          return rc;
      } else {
        if ((rc = c->cuda(lincomb(st, xp1, xp + t * n, 0.5 * dt, s.va, 0.5 * dt, s.vc, n), "heun"))) return rc;
        if ((rc = c->cuda(lincomb(st, xm1, xm + t * n, 0.5 * dt, s.vb, 0.5 * dt, s.vd, n), "heun"))) return rc;
      }
      c->launches += 2;
    }
  }
  return GBK_OK;
}

}  // namespace gbk

using namespace gbk;

// Scratch for the stand-alone entry points: four n x d temporaries and a flag in ctx->tmp.
static int deform_scratch(gbk_ctx *c, long rows, int d, DeformScratch *s) {
  size_t per = ((size_t)std::max(rows, 1L) * d * sizeof(double) + 255) & ~(size_t)255;
  int rc = c->ensure(c->tmp, 4 * per + 256, "deformation scratch");
  if (rc) return rc;
  char *b = (char *)c->tmp.p;
  s->va = (double *)b;
  s->vb = (double *)(b + per);
  s->vc = (double *)(b + 2 * per);
  s->vd = (double *)(b + 3 * per);
  s->flag = (int *)(b + 4 * per);
  return GBK_OK;
}

#define GBK_GUARD2(ctx)                                                      \
  do {                                                                       \
    if (!(ctx)) return GBK_ERR_ARG;                                          \
    (ctx)->err.clear();                                                      \
    if (cudaSetDevice((ctx)->device) != cudaSuccess) {                       \
      cudaGetLastError();                                                    \
      return (ctx)->fail(GBK_ERR_CUDA, "cudaSetDevice(%d)", (ctx)->device);  \
    }                                                                        \
  } while (0)

static int check_traj(gbk_ctx *c, int d, long ncp, int T) {
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "dimension %d not supported", d);
  if (ncp <= 0) return c->fail(GBK_ERR_ARG, "need at least one control point");
  if (T < 2) return c->fail(GBK_ERR_ARG, "need at least two time points (T=%d)", T);
  return GBK_OK;
}

extern "C" {

int gbk_shoot(gbk_ctx *c, int d, long ncp, const double *cp0, const double *mom0, int T,
              double sigma, double *pos_traj, double *mom_traj) {
  GBK_GUARD2(c);
  GBK_RANGE();
  if (int rc = check_traj(c, d, ncp, T)) return rc;
  if (!cp0 || !mom0 || !pos_traj || !mom_traj) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const long n = ncp * d;
  const double *dcp = io.in(cp0, n, "cp0");
  const double *dmo = io.in(mom0, n, "mom0");
  double *dpos = io.out(pos_traj, (size_t)T * n, "pos_traj");
  double *dmom = io.out(mom_traj, (size_t)T * n, "mom_traj");
  if (io.rc) return io.rc;
  DeformScratch s;
  if (int rc = deform_scratch(c, ncp, d, &s)) return rc;
  if (int rc = shoot_device(c, d, ncp, dcp, dmo, T, sigma, dpos, dmom, s)) return rc;
  return io.finish();
}

int gbk_flow_landmarks(gbk_ctx *c, int d, long ncp, const double *pos_traj, const double *mom_traj,
                       int T, double sigma, long nlm, const double *lm0, int heun,
                       double *lm_traj) {
  GBK_GUARD2(c);
  GBK_RANGE();
  if (int rc = check_traj(c, d, ncp, T)) return rc;
  if (nlm < 0) return c->fail(GBK_ERR_ARG, "negative landmark count");
  if (!pos_traj || !mom_traj || (nlm && (!lm0 || !lm_traj))) return c->fail(GBK_ERR_ARG, "null pointer");
  if (nlm == 0) return GBK_OK;
  HostIO io(c);
  const long n = ncp * d, m = nlm * d;
  const double *dpos = io.in(pos_traj, (size_t)T * n, "pos_traj");
  const double *dmom = io.in(mom_traj, (size_t)T * n, "mom_traj");
  const double *dl0 = io.in(lm0, m, "lm0");
  double *dlm = io.out(lm_traj, (size_t)T * m, "lm_traj");
  if (io.rc) return io.rc;
  DeformScratch s;
  if (int rc = deform_scratch(c, std::max(ncp, nlm), d, &s)) return rc;
  if (int rc = flow_device(c, d, ncp, dpos, dmom, T, sigma, nlm, dl0, heun, dlm, s)) return rc;
  return io.finish();
}

int gbk_adjoint_landmarks(gbk_ctx *c, int d, long ncp, const double *pos_traj,
                          const double *mom_traj, int T, double sigma, long nlm,
                          const double *lm_traj, const double *theta_final, int heun,
                          double *theta_traj) {
  GBK_GUARD2(c);
  GBK_RANGE();
  if (int rc = check_traj(c, d, ncp, T)) return rc;
  if (nlm <= 0) return c->fail(GBK_ERR_ARG, "need at least one landmark");
  if (!pos_traj || !mom_traj || !lm_traj || !theta_final || !theta_traj)
    return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const long n = ncp * d, m = nlm * d;
  const double *dpos = io.in(pos_traj, (size_t)T * n, "pos_traj");
  const double *dmom = io.in(mom_traj, (size_t)T * n, "mom_traj");
  const double *dlm = io.in(lm_traj, (size_t)T * m, "lm_traj");
  const double *dth = io.in(theta_final, m, "theta_final");
  double *dtt = io.out(theta_traj, (size_t)T * m, "theta_traj");
  if (io.rc) return io.rc;
  DeformScratch s;
  if (int rc = deform_scratch(c, std::max(ncp, nlm), d, &s)) return rc;
  if (int rc = adjoint_landmarks_device(c, d, ncp, dpos, dmom, T, sigma, nlm, dlm, dth, heun, dtt, s)) return rc;
  return io.finish();
}

int gbk_compute_update_at(gbk_ctx *c, int d, long ncp, const double *pos, const double *mom,
                          const double *xi_pos, const double *xi_mom, long nlm, const double *lm,
                          const double *theta, double sigma, double *dpos, double *dmom) {
  GBK_GUARD2(c);
  GBK_RANGE();
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "dimension %d not supported", d);
  if (ncp <= 0 || nlm < 0) return c->fail(GBK_ERR_ARG, "bad point counts");
  if (!pos || !mom || !xi_pos || !xi_mom || !dpos || !dmom || (nlm && (!lm || !theta)))
    return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const long n = ncp * d, m = nlm * d;
  const double *dp = io.in(pos, n, "pos"), *dm = io.in(mom, n, "mom");
  const double *dxp = io.in(xi_pos, n, "xi_pos"), *dxm = io.in(xi_mom, n, "xi_mom");
  const double *dl = io.in(lm, m, "lm"), *dt = io.in(theta, m, "theta");
  double *o0 = io.out(dpos, n, "dpos"), *o1 = io.out(dmom, n, "dmom");
  if (io.rc) return io.rc;
  if (int rc = update_at_device(c, d, ncp, dp, dm, dxp, dxm, nlm, dl, dt, sigma, o0, o1)) return rc;
  return io.finish();
}

int gbk_adjoint_diffeo(gbk_ctx *c, int d, long ncp, const double *pos_traj, const double *mom_traj,
                       int T, double sigma, long nlm, const double *lm_traj,
                       const double *theta_traj, int heun, double *xipos_traj,
                       double *ximom_traj) {
  GBK_GUARD2(c);
  GBK_RANGE();
  if (int rc = check_traj(c, d, ncp, T)) return rc;
  if (nlm < 0) return c->fail(GBK_ERR_ARG, "negative landmark count");
  if (!pos_traj || !mom_traj || !xipos_traj || !ximom_traj || (nlm && (!lm_traj || !theta_traj)))
    return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const long n = ncp * d, m = nlm * d;
  const double *dpos = io.in(pos_traj, (size_t)T * n, "pos_traj");
  const double *dmom = io.in(mom_traj, (size_t)T * n, "mom_traj");
  const double *dlm = io.in(lm_traj, (size_t)T * m, "lm_traj");
  const double *dth = io.in(theta_traj, (size_t)T * m, "theta_traj");
  double *dxp = io.out(xipos_traj, (size_t)T * n, "xipos_traj");
  double *dxm = io.out(ximom_traj, (size_t)T * n, "ximom_traj");
  if (io.rc) return io.rc;
  DeformScratch s;
  if (int rc = deform_scratch(c, ncp, d, &s)) return rc;
  if (int rc = adjoint_diffeo_device(c, d, ncp, dpos, dmom, T, sigma, nlm, dlm, dth, heun, dxp, dxm, s)) return rc;
  return io.finish();
}

}  // extern "C"
