// Currents and varifold data terms between two triangle meshes, with the gradient with respect to
// the vertices of the first (deformed) mesh.
//
// Currents (OrientedSurfaceMesh.cxx:124-352): faces carry centres c and normals
// n = (p2 - p0) x (p1 - p0) / 2. Varifolds (NonOrientedSurfaceMesh.cxx:124-378): n~ = n /
// sqrt(|n| + 1e-20) and the six products n~_p n~_q (p <= q). With the dual weights
// w(n~) = (n~0^2, 2 n~0 n~1, 2 n~0 n~2, n~1^2, 2 n~1 n~2, n~2^2) every varifold scalar
// n~^T M(v) n~ of the reference (special_product, :364-378) is the dot product v . w(n~), so
//   |S|^2 = sum_f w_f . (K MN)_f ,   <S,T> = sum_f w_f . (K_ST MN_T)_f
// and the varlin gradient the reference contracts face by face (:206-251) is the alpha-gradient
// with alpha = w. Each data term is therefore two fused pair passes (Convolve + alpha-gradient,
// sources S then T) plus FP64 face and vertex kernels; the target norm is one Convolve pass. The
// scatter of face terms to vertices (:210-237, :226-254) is a deterministic gather over a CSR
// vertex -> (face, corner) list: no atomics, bitwise reproducible.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_dispatch.h"
#include "gbk_geometry.h"
#include "gbk_hostio.h"
#include "gbk_ops.h"

namespace gbk {

static unsigned nblk(long n, int bs = 256) { return (unsigned)std::max(1L, (n + bs - 1) / bs); }

// centres, normals (currents) or centres, n~, MN, w (varifold)
__global__ void face_kernel(const double *pts, const int *tris, long nf, int kind, double *c,
                            double *n, double *mn, double *w) {
  long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const int i0 = tris[3 * f], i1 = tris[3 * f + 1], i2 = tris[3 * f + 2];
  double p0[3], p1[3], p2[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    p0[k] = pts[3 * i0 + k];
    p1[k] = pts[3 * i1 + k];
    p2[k] = pts[3 * i2 + k];
  }
  const double a[3] = {p2[0] - p0[0], p2[1] - p0[1], p2[2] - p0[2]};
  const double b[3] = {p1[0] - p0[0], p1[1] - p0[1], p1[2] - p0[2]};
  double nn[3] = {0.5 * (a[1] * b[2] - a[2] * b[1]), 0.5 * (a[2] * b[0] - a[0] * b[2]),
                  0.5 * (a[0] * b[1] - a[1] * b[0])};
#pragma unroll
  for (int k = 0; k < 3; ++k) c[3 * f + k] = (p0[k] + p1[k] + p2[k]) / 3.0;
  if (kind == 1) {
    const double s = 1.0 / sqrt(sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]) + 1e-20);
#pragma unroll
    for (int k = 0; k < 3; ++k) nn[k] *= s;
    mn[6 * f + 0] = nn[0] * nn[0];
    mn[6 * f + 1] = nn[0] * nn[1];
    mn[6 * f + 2] = nn[0] * nn[2];
    mn[6 * f + 3] = nn[1] * nn[1];
    mn[6 * f + 4] = nn[1] * nn[2];
    mn[6 * f + 5] = nn[2] * nn[2];
    w[6 * f + 0] = nn[0] * nn[0];
    w[6 * f + 1] = 2.0 * nn[0] * nn[1];
    w[6 * f + 2] = 2.0 * nn[0] * nn[2];
    w[6 * f + 3] = nn[1] * nn[1];
    w[6 * f + 4] = 2.0 * nn[1] * nn[2];
    w[6 * f + 5] = nn[2] * nn[2];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) n[3 * f + k] = nn[k];
}

// symmetric 3x3 from (00, 01, 02, 11, 12, 22) times x
__device__ inline void sym6_mul(const double *m, const double *x, double *y) {
  y[0] = m[0] * x[0] + m[1] * x[1] + m[2] * x[2];
  y[1] = m[1] * x[0] + m[3] * x[1] + m[4] * x[2];
  y[2] = m[2] * x[0] + m[4] * x[1] + m[5] * x[2];
}

// per-face vectors of the gradient: kt (crossed with the opposite edges) and gk (added to all
// three vertices)
__global__ void face_grad_kernel(long nf, int kind, const double *n, const double *mn,
                                 const double *kts, const double *ktt, const double *gs,
                                 const double *gt, double *kt, double *gk) {
  long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  if (kind == 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      kt[3 * f + k] = kts[3 * f + k] - ktt[3 * f + k];
      gk[3 * f + k] = (gs[3 * f + k] - gt[3 * f + k]) * 2.0 / 3.0;
    }
    return;
  }
  const double *nf3 = n + 3 * f;
  const double mag2 = nf3[0] * nf3[0] + nf3[1] * nf3[1] + nf3[2] * nf3[2];
  if (!(mag2 > 1e-20)) {  // NonOrientedSurfaceMesh.cxx:220
#pragma unroll
    for (int k = 0; k < 3; ++k) kt[3 * f + k] = gk[3 * f + k] = 0.0;
    return;
  }
  double dk[6], v[3], aux[3];
#pragma unroll
  for (int k = 0; k < 6; ++k) dk[k] = kts[6 * f + k] - ktt[6 * f + k];
  sym6_mul(dk, nf3, v);
#pragma unroll
  for (int k = 0; k < 3; ++k) v[k] *= 2.0;
  sym6_mul(mn + 6 * f, v, aux);
  const double inv = 1.0 / sqrt(mag2);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    kt[3 * f + k] = (v[k] - aux[k] / (2.0 * mag2)) * inv;
    gk[3 * f + k] = (gs[3 * f + k] - gt[3 * f + k]) * (2.0 / 3.0);
  }
}

// grad_v = sum over (face, corner) incident to v of e_corner x kt_f + gk_f, in CSR order
__global__ void vertex_gather_kernel(long nv, const double *pts, const int *tris, const int *ptr,
                                     const int *fc, const double *kt, const double *gk,
                                     double *grad, double scale, int accumulate) {
  long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double g[3] = {0.0, 0.0, 0.0};
  for (int q = ptr[v]; q < ptr[v + 1]; ++q) {
    const int f = fc[q] / 3, corner = fc[q] % 3;
    const int a = tris[3 * f + (corner + 2) % 3], b = tris[3 * f + (corner + 1) % 3];
    // e0 = p2 - p1, e1 = p0 - p2, e2 = p1 - p0: e_corner = p[corner-1] - p[corner+1]
    double e[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) e[k] = pts[3 * a + k] - pts[3 * b + k];
    const double *t = kt + 3 * f;
    g[0] += e[1] * t[2] - e[2] * t[1] + gk[3 * f + 0];
    g[1] += e[2] * t[0] - e[0] * t[2] + gk[3 * f + 1];
    g[2] += e[0] * t[1] - e[1] * t[0] + gk[3 * f + 2];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) grad[3 * v + k] = accumulate ? grad[3 * v + k] + scale * g[k] : scale * g[k];
}

// ---------------------------------------------------------------------------------------------
// SurfaceTerm
// ---------------------------------------------------------------------------------------------
static int dalloc(gbk_ctx *c, void **p, size_t bytes, std::vector<void *> &owned) {
  if (bytes == 0) bytes = 8;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return c->cuda(e, "cudaMalloc (surface term)");
  owned.push_back(*p);
  return GBK_OK;
}

void build_csr(long nv, long nf, const int *tris, std::vector<int> &ptr, std::vector<int> &fc) {
  ptr.assign(nv + 1, 0);
  for (long q = 0; q < 3 * nf; ++q) ptr[tris[q] + 1]++;
  for (long v = 0; v < nv; ++v) ptr[v + 1] += ptr[v];
  fc.assign(3 * nf, 0);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (long q = 0; q < 3 * nf; ++q) fc[fill[tris[q]]++] = (int)q;  // face * 3 + corner, face order
}

int SurfaceTerm::init(gbk_ctx *c, int kind_, double sigma_, long nv_, long nf_, const int *tris_h,
                      long nv_t_, long nf_t_, const int *tris_t_h) {
  kind = kind_;
  sigma = sigma_;
  nv = nv_;
  nf = nf_;
  nv_t = nv_t_;
  nf_t = nf_t_;
  dw = kind == 1 ? 6 : 3;
  for (long q = 0; q < 3 * nf; ++q)
    if (tris_h[q] < 0 || tris_h[q] >= nv) return c->fail(GBK_ERR_ARG, "triangle index %d out of range", tris_h[q]);
  for (long q = 0; q < 3 * nf_t; ++q)
    if (tris_t_h[q] < 0 || tris_t_h[q] >= nv_t) return c->fail(GBK_ERR_ARG, "target triangle index out of range");
  std::vector<int> ptr, fc;
  build_csr(nv, nf, tris_h, ptr, fc);
  int rc;
  const size_t F3 = (size_t)nf * 3 * sizeof(double), FW = (size_t)nf * dw * sizeof(double);
  const size_t T3 = (size_t)nf_t * 3 * sizeof(double), TW = (size_t)nf_t * dw * sizeof(double);
  if ((rc = dalloc(c, (void **)&tris, (size_t)nf * 3 * sizeof(int), owned))) return rc;
  if ((rc = dalloc(c, (void **)&tris_t, (size_t)nf_t * 3 * sizeof(int), owned))) return rc;
  if ((rc = dalloc(c, (void **)&csr_ptr, (size_t)(nv + 1) * sizeof(int), owned))) return rc;
  if ((rc = dalloc(c, (void **)&csr_fc, (size_t)nf * 3 * sizeof(int), owned))) return rc;
  double **f3[] = {&cs, &ns, &gs, &gt, &kt, &gk};
  for (double **p : f3)
    if ((rc = dalloc(c, (void **)p, F3, owned))) return rc;
  double **fw[] = {&mns, &ws, &kts, &ktt};
  for (double **p : fw)
    if ((rc = dalloc(c, (void **)p, FW, owned))) return rc;
  double **t3[] = {&ct, &nt};
  for (double **p : t3)
    if ((rc = dalloc(c, (void **)p, T3, owned))) return rc;
  double **tw[] = {&mnt, &wt, &kttt};
  for (double **p : tw)
    if ((rc = dalloc(c, (void **)p, TW, owned))) return rc;
  if ((rc = dalloc(c, (void **)&scal, 8 * sizeof(double), owned))) return rc;
  cudaStream_t st = c->stream;
  if ((rc = c->cuda(cudaMemcpyAsync(tris, tris_h, (size_t)nf * 3 * sizeof(int), cudaMemcpyHostToDevice, st), "H2D"))) return rc;
  if ((rc = c->cuda(cudaMemcpyAsync(tris_t, tris_t_h, (size_t)nf_t * 3 * sizeof(int), cudaMemcpyHostToDevice, st), "H2D"))) return rc;
  if ((rc = c->cuda(cudaMemcpyAsync(csr_ptr, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice, st), "H2D"))) return rc;
  if ((rc = c->cuda(cudaMemcpyAsync(csr_fc, fc.data(), fc.size() * sizeof(int), cudaMemcpyHostToDevice, st), "H2D"))) return rc;
  return c->cuda(cudaStreamSynchronize(st), "sync");  // host vectors die here
}

void SurfaceTerm::release() {
  for (void *p : owned) cudaFree(p);
  owned.clear();
}

// Target: faces and |T|^2 (stored in scal[0]); done once per target.
int SurfaceTerm::set_target(gbk_ctx *c, const double *pts_t) {
  cudaStream_t st = c->stream;
  face_kernel<<<nblk(nf_t), 256, 0, st>>>(pts_t, tris_t, nf_t, kind, ct, nt, mnt, wt);
  int rc = c->cuda(cudaGetLastError(), "face_kernel");
  if (rc) return rc;
  c->launches += 1;
  PairArgs a = pair_args(nf_t, nf_t, sigma);
  a.x = ct;
  a.y = ct;
  a.w = kind ? mnt : nt;
  a.w_ld = dw;
  a.out0 = kttt;
  a.out0_ld = dw;
  if ((rc = c->launch(OP_CONV, 3, dw, a))) return rc;
  if ((rc = c->cuda(dot_f64(st, kind ? wt : nt, kttt, nf_t * dw, scal + 0, 0), "dot"))) return rc;
  c->launches += 1;
  return GBK_OK;
}

// match = |T|^2 + |S|^2 - 2 <S,T> into match_dev (device double); if grad_dev is not null,
// grad_dev (+)= scale * d match / d vertices.
int SurfaceTerm::evaluate(gbk_ctx *c, const double *pts_s, double *match_dev, double *grad_dev,
                          double scale, int accumulate) {
  cudaStream_t st = c->stream;
  face_kernel<<<nblk(nf), 256, 0, st>>>(pts_s, tris, nf, kind, cs, ns, mns, ws);
  int rc = c->cuda(cudaGetLastError(), "face_kernel");
  if (rc) return rc;
  c->launches += 1;
  const double *alpha = kind ? ws : ns;
  const double *wsrc = kind ? mns : ns;
  const int op = grad_dev ? OP_CONV_GRADA : OP_CONV;
  // self pass: (K W_S)(c_S) and its alpha-gradient
  PairArgs a = pair_args(nf, nf, sigma);
  a.x = cs;
  a.ta = alpha;
  a.ta_ld = dw;
  a.y = cs;
  a.w = wsrc;
  a.w_ld = dw;
  a.out0 = kts;
  a.out0_ld = dw;
  a.out1 = gs;
  a.out1_ld = 3;
  if ((rc = c->launch(op, 3, dw, a))) return rc;
  // cross pass: (K W_T)(c_S) and its alpha-gradient
  PairArgs b = a;
  b.ny = nf_t;
  b.y = ct;
  b.w = kind ? mnt : nt;
  b.out0 = ktt;
  b.out1 = gt;
  if ((rc = c->launch(op, 3, dw, b))) return rc;
  // match = |T|^2 + w_S . K_SS W_S - 2 w_S . K_ST W_T (w_S = n_S for currents)
  if ((rc = c->cuda(dot_f64(st, alpha, kts, nf * dw, scal + 1, 0), "dot"))) return rc;
  if ((rc = c->cuda(dot_f64(st, alpha, ktt, nf * dw, scal + 2, 0), "dot"))) return rc;
  if ((rc = c->cuda(scalar_combine(st, match_dev, scal + 0, 1.0, scal + 1, 1.0, scal + 2, -2.0), "combine"))) return rc;
  c->launches += 3;
  if (!grad_dev) return GBK_OK;
  face_grad_kernel<<<nblk(nf), 256, 0, st>>>(nf, kind, ns, mns, kts, ktt, gs, gt, kt, gk);
  if ((rc = c->cuda(cudaGetLastError(), "face_grad_kernel"))) return rc;
  vertex_gather_kernel<<<nblk(nv), 256, 0, st>>>(nv, pts_s, tris, csr_ptr, csr_fc, kt, gk, grad_dev,
                                                  scale, accumulate);
  c->launches += 2;
  return c->cuda(cudaGetLastError(), "vertex_gather_kernel");
}

}  // namespace gbk

using namespace gbk;

static int surface_match(gbk_ctx *c, int kind, long nv, const double *pts, long nf, const int *tris,
                         long nv_t, const double *pts_t, long nf_t, const int *tris_t, double sigma,
                         double *match, double *grad) {
  if (!c) return GBK_ERR_ARG;
  c->err.clear();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (nv <= 0 || nf <= 0 || nv_t <= 0 || nf_t <= 0) return c->fail(GBK_ERR_ARG, "empty mesh");
  if (!pts || !tris || !pts_t || !tris_t || !match) return c->fail(GBK_ERR_ARG, "null pointer");
  if (c->capturing()) return c->fail(GBK_ERR_STATE, "the stand-alone data term allocates; use a registration object under capture");
  // triangles are needed on the host for the vertex -> face lists
  std::vector<int> th((size_t)nf * 3), tth((size_t)nf_t * 3);
  cudaMemcpy(th.data(), tris, th.size() * sizeof(int), cudaMemcpyDefault);
  cudaMemcpy(tth.data(), tris_t, tth.size() * sizeof(int), cudaMemcpyDefault);
  if (int rc = c->cuda(cudaGetLastError(), "copy triangles")) return rc;
  SurfaceTerm s;
  int rc = s.init(c, kind, sigma, nv, nf, th.data(), nv_t, nf_t, tth.data());
  if (!rc) {
    HostIO io(c);
    const double *dp = io.in(pts, (size_t)nv * 3, "pts");
    const double *dpt = io.in(pts_t, (size_t)nv_t * 3, "pts_t");
    double *dm = io.out(match, 1, "match");
    double *dg = io.out(grad, grad ? (size_t)nv * 3 : 0, "grad");
    rc = io.rc;
    if (!rc) rc = s.set_target(c, dpt);
    if (!rc) rc = s.evaluate(c, dp, dm, dg, 1.0, 0);
    if (!rc) rc = io.finish();
    if (!rc) rc = c->cuda(cudaStreamSynchronize(c->stream), "sync");
  }
  cudaStreamSynchronize(c->stream);
  s.release();
  return rc;
}

extern "C" {

int gbk_currents_match(gbk_ctx *c, long nv, const double *pts, long nf, const int *tris, long nv_t,
                       const double *pts_t, long nf_t, const int *tris_t, double sigma,
                       double *match, double *grad) {
  return surface_match(c, 0, nv, pts, nf, tris, nv_t, pts_t, nf_t, tris_t, sigma, match, grad);
}

int gbk_varifold_match(gbk_ctx *c, long nv, const double *pts, long nf, const int *tris, long nv_t,
                       const double *pts_t, long nf_t, const int *tris_t, double sigma,
                       double *match, double *grad) {
  return surface_match(c, 1, nv, pts, nf, tris, nv_t, pts_t, nf_t, tris_t, sigma, match, grad);
}

}  // extern "C"
