// Data terms between a deformed object and a fixed target, with the gradient with respect to the
// vertices of the deformed one: currents and varifolds of triangle meshes (d = 3) and polylines
// (d = 2, 3), scalar measures of weighted point clouds and volume meshes, and landmarks.
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
//
// Scalar measures (PointCloud.cxx:104-254, OrientedVolumeMesh.cxx:115-367) are the same two pair
// passes with one weight column: the point weights, or the cell volumes |det| / d! at the cell
// centres. Landmarks (Landmark.cxx:288-322) need no kernel sum.
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

// Cells of CELL vertices in D dimensions: triangles (CELL 3, D 3) carry centres and normals
// n = (p2 - p0) x (p1 - p0) / 2; segments (CELL 2) centres and tangents t = p1 - p0
// (OrientedPolyLine::UpdateCentersTangents). Varifolds (kind 1) use v~ = v / sqrt(|v| + 1e-20),
// the D(D+1)/2 upper-triangle products MN and the dual weights w (off-diagonal entries doubled).
template <int D, int CELL>
__global__ void cell_kernel(const double *pts, const int *cells, long nf, int kind, double *c, double *n,
                            double *mn, double *w) {
  pdl_entry();
  constexpr int NM = D * (D + 1) / 2;
  long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  double p[CELL][D];
#pragma unroll
  for (int q = 0; q < CELL; ++q)
#pragma unroll
    for (int k = 0; k < D; ++k) p[q][k] = pts[(long)D * cells[CELL * f + q] + k];
  double v[D];
  if constexpr (CELL == 3) {
    static_assert(D == 3, "triangles live in 3-D");
    const double a[3] = {p[2][0] - p[0][0], p[2][1] - p[0][1], p[2][2] - p[0][2]};
    const double b[3] = {p[1][0] - p[0][0], p[1][1] - p[0][1], p[1][2] - p[0][2]};
    v[0] = 0.5 * (a[1] * b[2] - a[2] * b[1]);
    v[1] = 0.5 * (a[2] * b[0] - a[0] * b[2]);
    v[2] = 0.5 * (a[0] * b[1] - a[1] * b[0]);
#pragma unroll
    for (int k = 0; k < 3; ++k) c[3 * f + k] = (p[0][k] + p[1][k] + p[2][k]) / 3.0;
  } else {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      v[k] = p[1][k] - p[0][k];
      c[D * f + k] = (p[0][k] + p[1][k]) / 2.0;
    }
  }
  if (kind == 1) {
    double m2 = 0.0;
#pragma unroll
    for (int k = 0; k < D; ++k) m2 += v[k] * v[k];
    const double s = 1.0 / sqrt(sqrt(m2) + 1e-20);
#pragma unroll
    for (int k = 0; k < D; ++k) v[k] *= s;
    int q = 0;
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
      for (int b = a; b < D; ++b, ++q) {
        mn[NM * f + q] = v[a] * v[b];
        w[NM * f + q] = (a == b ? 1.0 : 2.0) * v[a] * v[b];
      }
  }
#pragma unroll
  for (int k = 0; k < D; ++k) n[D * f + k] = v[k];
}

// symmetric D x D from its upper triangle (row by row) times x
template <int D>
__device__ inline void sym_mul(const double *m, const double *x, double *y) {
  double S[D][D];
  int q = 0;
#pragma unroll
  for (int a = 0; a < D; ++a)
#pragma unroll
    for (int b = a; b < D; ++b, ++q) S[a][b] = S[b][a] = m[q];
#pragma unroll
  for (int a = 0; a < D; ++a) {
    y[a] = 0.0;
#pragma unroll
    for (int b = 0; b < D; ++b) y[a] += S[a][b] * x[b];
  }
}

// Per-cell vectors of the gradient. Triangles: kt (crossed with the opposite edges) and gk (added
// to all three vertices): OrientedSurfaceMesh.cxx:165-241, NonOrientedSurfaceMesh.cxx:169-265.
// Segments: kt (minus at the first end, plus at the second) and gk (added to both ends):
// OrientedPolyLine::ComputeMatchGradient, NonOrientedPolyLine.cxx:174-256.
template <int D, int CELL>
__global__ void cell_grad_kernel(long nf, int kind, const double *n, const double *mn, const double *kts,
                                 const double *ktt, const double *gs, const double *gt, double *kt, double *gk) {
  pdl_entry();
  constexpr int NM = D * (D + 1) / 2;
  long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  const double gscale = CELL == 3 ? 2.0 / 3.0 : 1.0;  // d centre / d vertex, times 2
  if (kind == 0) {
#pragma unroll
    for (int k = 0; k < D; ++k) {
      kt[D * f + k] = (CELL == 3 ? 1.0 : 2.0) * (kts[D * f + k] - ktt[D * f + k]);
      gk[D * f + k] = (gs[D * f + k] - gt[D * f + k]) * gscale;
    }
    return;
  }
  const double *nv = n + D * f;
  double mag2 = 0.0;
#pragma unroll
  for (int k = 0; k < D; ++k) mag2 += nv[k] * nv[k];
  if (!(mag2 > 1e-20)) {
#pragma unroll
    for (int k = 0; k < D; ++k) kt[D * f + k] = gk[D * f + k] = 0.0;
    return;
  }
  double dk[NM], v[D], aux[D];
#pragma unroll
  for (int k = 0; k < NM; ++k) dk[k] = kts[NM * f + k] - ktt[NM * f + k];
  sym_mul<D>(dk, nv, v);
#pragma unroll
  for (int k = 0; k < D; ++k) v[k] *= (CELL == 3 ? 2.0 : 4.0);
  sym_mul<D>(mn + NM * f, v, aux);
  const double inv = 1.0 / sqrt(mag2);
#pragma unroll
  for (int k = 0; k < D; ++k) {
    kt[D * f + k] = (v[k] - aux[k] / (2.0 * mag2)) * inv;
    gk[D * f + k] = (gs[D * f + k] - gt[D * f + k]) * gscale;
  }
}

// grad_v = sum over the (cell, corner) pairs of vertex v, in CSR order, of the cell's vector for
// that corner: e_corner x kt + gk for triangles, -/+ kt + gk for segments
template <int D, int CELL>
__global__ void vertex_gather_kernel(long nv, const double *pts, const int *cells, const int *ptr, const int *fc,
                                     const double *kt, const double *gk, double *grad, double scale,
                                     int accumulate) {
  pdl_entry();
  long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double g[D];
#pragma unroll
  for (int k = 0; k < D; ++k) g[k] = 0.0;
  for (int q = ptr[v]; q < ptr[v + 1]; ++q) {
    const int f = fc[q] / CELL, corner = fc[q] % CELL;
    const double *t = kt + D * f;
    if constexpr (CELL == 3) {
      const int a = cells[3 * f + (corner + 2) % 3], b = cells[3 * f + (corner + 1) % 3];
      // e0 = p2 - p1, e1 = p0 - p2, e2 = p1 - p0: e_corner = p[corner-1] - p[corner+1]
      double e[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) e[k] = pts[3 * a + k] - pts[3 * b + k];
      g[0] += e[1] * t[2] - e[2] * t[1] + gk[3 * f + 0];
      g[1] += e[2] * t[0] - e[0] * t[2] + gk[3 * f + 1];
      g[2] += e[0] * t[1] - e[1] * t[0] + gk[3 * f + 2];
    } else {
      const double sgn = corner == 0 ? -1.0 : 1.0;
#pragma unroll
      for (int k = 0; k < D; ++k) g[k] += sgn * t[k] + gk[D * f + k];
    }
  }
#pragma unroll
  for (int k = 0; k < D; ++k) grad[D * v + k] = accumulate ? grad[D * v + k] + scale * g[k] : scale * g[k];
}

// Scalar measures: centres and weights. Points (CELL 1) are their own centres and keep the weights
// stored at init; simplices (CELL = D + 1) take the mean of their vertices (summed in order) and
// |det(p_1 - p_0, ..., p_D - p_0)| / D! (OrientedVolumeMesh::UpdateCentersNormals, :299-335), with
// the determinant's sign into sg when it is given.
template <int D, int CELL>
__global__ void measure_kernel(const double *pts, const int *cells, long nf, double *c, double *w, double *sg) {
  pdl_entry();
  long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  if constexpr (CELL == 1) {
#pragma unroll
    for (int k = 0; k < D; ++k) c[D * f + k] = pts[D * f + k];
  } else {
    static_assert(CELL == D + 1, "volume cells are simplices");
    double p[CELL][D];
#pragma unroll
    for (int q = 0; q < CELL; ++q)
#pragma unroll
      for (int k = 0; k < D; ++k) p[q][k] = pts[(long)D * cells[CELL * f + q] + k];
    double e[D][D];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      double s = p[0][k];
#pragma unroll
      for (int q = 1; q < CELL; ++q) s += p[q][k];
      c[D * f + k] = s / (D + 1.0);
#pragma unroll
      for (int q = 1; q < CELL; ++q) e[q - 1][k] = p[q][k] - p[0][k];
    }
    double det;
    if constexpr (D == 3)
      det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) - e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
            e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
    else
      det = e[0][0] * e[1][1] - e[0][1] * e[1][0];
    w[f] = fabs(det) / (D == 3 ? 6.0 : 2.0);
    if (sg) sg[f] = det < 0.0 ? -1.0 : 1.0;
  }
}

// Per-cell gradient parts of a scalar measure. Points: gk = 2 (G_S + G_T) as PointCloud.cxx:194
// (reference formula) or 2 (G_S - G_T) (exact). Volumes: kt = Ktau = (K_S V_S - K_T V_T)(c), times
// the determinant's sign when exact, and gk = (G_S - G_T) / ((D + 1) / 2) (OrientedVolumeMesh.cxx:
// 196-209).
template <int D, int CELL>
__global__ void measure_grad_kernel(long nf, int exact, const double *kts, const double *ktt, const double *gs,
                                    const double *gt, const double *sg, double *kt, double *gk) {
  pdl_entry();
  long f = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nf) return;
  if constexpr (CELL == 1) {
#pragma unroll
    for (int k = 0; k < D; ++k)
      gk[D * f + k] = exact ? (gs[D * f + k] - gt[D * f + k]) * 2.0 : (gs[D * f + k] + gt[D * f + k]) * 2.0;
  } else {
    const double ktau = kts[f] - ktt[f];
    kt[f] = exact ? ktau * sg[f] : ktau;
#pragma unroll
    for (int k = 0; k < D; ++k) gk[D * f + k] = (gs[D * f + k] - gt[D * f + k]) / ((D + 1.0) / 2.0);
  }
}

// d det / d p_corner of a simplex, written per corner as OrientedVolumeMesh::ComputeMatchGradient
// does (:214-227 in 3-D: v0 = (p3 - p1) x (p2 - p1), v1 = (p2 - p0) x (p3 - p0),
// v2 = (p3 - p0) x (p1 - p0), v3 = (p1 - p0) x (p2 - p0); :254-266 in 2-D)
template <int D>
__device__ inline void simplex_corner(const double *pts, const int *cv, int corner, double *v) {
  auto P = [&](int q, int k) { return pts[(long)D * cv[q] + k]; };
  if constexpr (D == 3) {
    int o, a, b;  // v = (p_a - p_o) x (p_b - p_o)
    switch (corner) {
      case 0: o = 1, a = 3, b = 2; break;
      case 1: o = 0, a = 2, b = 3; break;
      case 2: o = 0, a = 3, b = 1; break;
      default: o = 0, a = 1, b = 2; break;
    }
    const double x[3] = {P(a, 0) - P(o, 0), P(a, 1) - P(o, 1), P(a, 2) - P(o, 2)};
    const double y[3] = {P(b, 0) - P(o, 0), P(b, 1) - P(o, 1), P(b, 2) - P(o, 2)};
    v[0] = x[1] * y[2] - x[2] * y[1];
    v[1] = x[2] * y[0] - x[0] * y[2];
    v[2] = x[0] * y[1] - x[1] * y[0];
  } else {
    const int a = (corner + 1) % 3, b = (corner + 2) % 3;  // v = (p_a,y - p_b,y, p_b,x - p_a,x)
    v[0] = P(a, 1) - P(b, 1);
    v[1] = P(b, 0) - P(a, 0);
  }
}

// grad_v of a scalar measure: points take their own gk; simplex vertices sum, over their (cell,
// corner) pairs in CSR (cell) order, c_D v_corner Ktau and then gk, with c_3 = 1.0f / 3.0f as the
// reference writes it in single precision and c_2 = 1
template <int D, int CELL>
__global__ void measure_gather_kernel(long nv, const double *pts, const int *cells, const int *ptr, const int *fc,
                                      const double *kt, const double *gk, double *grad, double scale,
                                      int accumulate) {
  pdl_entry();
  long v = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  double g[D];
  if constexpr (CELL == 1) {
#pragma unroll
    for (int k = 0; k < D; ++k) g[k] = gk[D * v + k];
  } else {
    const double third = (double)(1.0f / 3.0f);
#pragma unroll
    for (int k = 0; k < D; ++k) g[k] = 0.0;
    for (int q = ptr[v]; q < ptr[v + 1]; ++q) {
      const int f = fc[q] / CELL, corner = fc[q] % CELL;
      double u[D];
      simplex_corner<D>(pts, cells + (long)CELL * f, corner, u);
#pragma unroll
      for (int k = 0; k < D; ++k) {
        g[k] += D == 3 ? third * u[k] * kt[f] : u[k] * kt[f];
        g[k] += gk[D * f + k];
      }
    }
  }
#pragma unroll
  for (int k = 0; k < D; ++k) grad[D * v + k] = accumulate ? grad[D * v + k] + scale * g[k] : scale * g[k];
}

__global__ void fill_kernel(double *p, long n, double v) {
  pdl_entry();
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

static cudaError_t fill_ones(cudaStream_t st, double *p, long n) {
  return launch(fill_kernel, nblk(n), 256, 0, st, p, n, 1.0);
}

// launches one of the measure kernels for the term's (d, cell); a launch error is left for
// cudaGetLastError
#define GBK_MEASURE_DISPATCH(T, KERNEL, GRID, ST, ...)                     \
  do {                                                                     \
    if ((T).cell == 1) {                                                   \
      if ((T).d == 2)                                                      \
        (void)launch(KERNEL<2, 1>, (GRID), 256, 0, (ST), __VA_ARGS__);     \
      else                                                                 \
        (void)launch(KERNEL<3, 1>, (GRID), 256, 0, (ST), __VA_ARGS__);     \
    } else if ((T).d == 2) {                                               \
      (void)launch(KERNEL<2, 3>, (GRID), 256, 0, (ST), __VA_ARGS__);       \
    } else {                                                               \
      (void)launch(KERNEL<3, 4>, (GRID), 256, 0, (ST), __VA_ARGS__);       \
    }                                                                      \
  } while (0)

// launches one of the cell kernels for the term's (d, cell); a launch error is left for
// cudaGetLastError
#define GBK_CELL_DISPATCH(T, KERNEL, GRID, ST, ...)                       \
  do {                                                                     \
    if ((T).cell == 3)                                                     \
      (void)launch(KERNEL<3, 3>, (GRID), 256, 0, (ST), __VA_ARGS__);       \
    else if ((T).d == 2)                                                   \
      (void)launch(KERNEL<2, 2>, (GRID), 256, 0, (ST), __VA_ARGS__);       \
    else                                                                   \
      (void)launch(KERNEL<3, 2>, (GRID), 256, 0, (ST), __VA_ARGS__);       \
  } while (0)

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

void build_csr(long nv, long nf, int cell, const int *cells, std::vector<int> &ptr, std::vector<int> &fc) {
  ptr.assign(nv + 1, 0);
  for (long q = 0; q < cell * nf; ++q) ptr[cells[q] + 1]++;
  for (long v = 0; v < nv; ++v) ptr[v + 1] += ptr[v];
  fc.assign(cell * nf, 0);
  std::vector<int> fill(ptr.begin(), ptr.end() - 1);
  for (long q = 0; q < cell * nf; ++q) fc[fill[cells[q]]++] = (int)q;  // cell * CELL + corner, cell order
}

int SurfaceTerm::init(gbk_ctx *c, int kind_, int d_, int cell_, double sigma_, long nv_, long nf_,
                      const int *tris_h, long nv_t_, long nf_t_, const int *tris_t_h, const double *w_h,
                      const double *w_t_h) {
  kind = kind_;
  d = d_;
  cell = cell_;
  sigma = sigma_;
  nv = nv_;
  nf = nf_;
  nv_t = nv_t_;
  nf_t = nf_t_;
  exact = c->gradient_mode == GBK_GRADIENT_EXACT;
  const bool ok = kind <= 1 ? ((d == 3 && cell == 3) || (d == 2 && cell == 2) || (d == 3 && cell == 2))
                            : (kind == 2 ? (d == 2 || d == 3) && (cell == 1 || cell == d + 1)
                                         : kind == 3 && (d == 2 || d == 3) && cell == 1);
  if (!ok) return c->fail(GBK_ERR_UNSUPPORTED, "data term %d of %d-vertex cells in %d dimensions", kind, cell, d);
  if (cell == 1 && (nf != nv || nf_t != nv_t)) return c->fail(GBK_ERR_ARG, "a point set has one cell per point");
  if (kind == 3 && nv != nv_t) return c->fail(GBK_ERR_ARG, "landmark objects need the same number of points");
  dw = kind == 1 ? d * (d + 1) / 2 : (kind >= 2 ? 1 : d);
  std::vector<int> ptr, fc;
  if (cell > 1) {
    for (long q = 0; q < cell * nf; ++q)
      if (tris_h[q] < 0 || tris_h[q] >= nv) return c->fail(GBK_ERR_ARG, "cell index %d out of range", tris_h[q]);
    for (long q = 0; q < cell * nf_t; ++q)
      if (tris_t_h[q] < 0 || tris_t_h[q] >= nv_t) return c->fail(GBK_ERR_ARG, "target cell index out of range");
    build_csr(nv, nf, cell, tris_h, ptr, fc);
  }
  int rc;
  const size_t F3 = (size_t)nf * d * sizeof(double), FW = (size_t)nf * dw * sizeof(double);
  const size_t T3 = (size_t)nf_t * d * sizeof(double), TW = (size_t)nf_t * dw * sizeof(double);
  if ((rc = dalloc(c, (void **)&tris, (size_t)nf * cell * sizeof(int), owned))) return rc;
  if ((rc = dalloc(c, (void **)&tris_t, (size_t)nf_t * cell * sizeof(int), owned))) return rc;
  if ((rc = dalloc(c, (void **)&csr_ptr, (size_t)(nv + 1) * sizeof(int), owned))) return rc;
  if ((rc = dalloc(c, (void **)&csr_fc, (size_t)nf * cell * sizeof(int), owned))) return rc;
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
  if ((rc = dalloc(c, (void **)&sg, (size_t)nf * sizeof(double), owned))) return rc;
  if ((rc = dalloc(c, (void **)&scal, 8 * sizeof(double), owned))) return rc;
  cudaStream_t st = c->stream;
  if (cell > 1) {
    if ((rc = c->cuda(cudaMemcpyAsync(tris, tris_h, (size_t)nf * cell * sizeof(int), cudaMemcpyHostToDevice, st), "H2D"))) return rc;
    if ((rc = c->cuda(cudaMemcpyAsync(tris_t, tris_t_h, (size_t)nf_t * cell * sizeof(int), cudaMemcpyHostToDevice, st), "H2D"))) return rc;
    if ((rc = c->cuda(cudaMemcpyAsync(csr_ptr, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice, st), "H2D"))) return rc;
    if ((rc = c->cuda(cudaMemcpyAsync(csr_fc, fc.data(), fc.size() * sizeof(int), cudaMemcpyHostToDevice, st), "H2D"))) return rc;
  }
  if (kind == 2 && cell == 1) {  // unit weights, then the given ones
    if ((rc = c->cuda(fill_ones(st, ns, nf), "fill"))) return rc;
    if ((rc = c->cuda(fill_ones(st, nt, nf_t), "fill"))) return rc;
    if (w_h && (rc = c->cuda(cudaMemcpyAsync(ns, w_h, (size_t)nf * sizeof(double), cudaMemcpyDefault, st), "weights"))) return rc;
    if (w_t_h && (rc = c->cuda(cudaMemcpyAsync(nt, w_t_h, (size_t)nf_t * sizeof(double), cudaMemcpyDefault, st), "weights"))) return rc;
  }
  return c->cuda(cudaStreamSynchronize(st), "sync");  // host vectors die here
}

int SurfaceTerm::set_weights(gbk_ctx *c, const double *w, const double *w_t) {
  if (!(kind == 2 && cell == 1)) return c->fail(GBK_ERR_STATE, "point weights belong to point clouds");
  cudaStream_t st = c->stream;
  int rc;
  if (w && (rc = c->cuda(cudaMemcpyAsync(ns, w, (size_t)nf * sizeof(double), cudaMemcpyDefault, st), "weights"))) return rc;
  if (w_t && (rc = c->cuda(cudaMemcpyAsync(nt, w_t, (size_t)nf_t * sizeof(double), cudaMemcpyDefault, st), "weights"))) return rc;
  if (tgt && (rc = set_target(c, tgt))) return rc;
  return c->cuda(cudaStreamSynchronize(st), "sync");
}

void SurfaceTerm::release() {
  for (void *p : owned) cudaFree(p);
  owned.clear();
}

// Target: faces and |T|^2 (stored in scal[0]); done once per target.
int SurfaceTerm::set_target(gbk_ctx *c, const double *pts_t) {
  cudaStream_t st = c->stream;
  tgt = pts_t;
  if (kind == 3) return c->cuda(cudaMemcpyAsync(ct, pts_t, (size_t)nv_t * d * sizeof(double), cudaMemcpyDefault, st), "copy");
  if (kind == 2)
    GBK_MEASURE_DISPATCH(*this, measure_kernel, nblk(nf_t), st, pts_t, tris_t, nf_t, ct, nt, nullptr);
  else
    GBK_CELL_DISPATCH(*this, cell_kernel, nblk(nf_t), st, pts_t, tris_t, nf_t, kind, ct, nt, mnt, wt);
  int rc = c->cuda(cudaGetLastError(), "cell_kernel");
  if (rc) return rc;
  c->launches += 1;
  PairArgs a = pair_args(nf_t, nf_t, sigma);
  a.x = ct;
  a.y = ct;
  a.w = kind == 1 ? mnt : nt;
  a.w_ld = dw;
  a.out0 = kttt;
  a.out0_ld = dw;
  if ((rc = c->launch(OP_CONV, d, dw, a))) return rc;
  if ((rc = c->cuda(dot_f64(st, kind == 1 ? wt : nt, kttt, nf_t * dw, scal + 0, 0), "dot"))) return rc;
  c->launches += 1;
  return GBK_OK;
}

// match = |T|^2 + |S|^2 - 2 <S,T> into match_dev (device double); if grad_dev is not null,
// grad_dev (+)= scale * d match / d vertices.
int SurfaceTerm::evaluate(gbk_ctx *c, const double *pts_s, double *match_dev, double *grad_dev,
                          double scale, int accumulate) {
  cudaStream_t st = c->stream;
  int rc;
  if (kind == 3) {  // landmarks: |S - T|^2 and 2 (S - T)
    const long m = nv * d;
    if ((rc = c->cuda(lincomb(st, gk, pts_s, -1.0, ct, 0.0, nullptr, m), "difference"))) return rc;
    if ((rc = c->cuda(dot_f64(st, gk, gk, m, scal + 1, 0), "dot"))) return rc;
    if ((rc = c->cuda(scalar_combine(st, match_dev, scal + 1, 1.0, nullptr, 0.0, nullptr, 0.0), "combine"))) return rc;
    c->launches += 3;
    if (!grad_dev) return GBK_OK;
    c->launches += 1;
    return c->cuda(lincomb(st, grad_dev, accumulate ? grad_dev : nullptr, 2.0 * scale, gk, 0.0, nullptr, m), "gradient");
  }
  if (kind == 2)
    GBK_MEASURE_DISPATCH(*this, measure_kernel, nblk(nf), st, pts_s, tris, nf, cs, ns, sg);
  else
    GBK_CELL_DISPATCH(*this, cell_kernel, nblk(nf), st, pts_s, tris, nf, kind, cs, ns, mns, ws);
  rc = c->cuda(cudaGetLastError(), "cell_kernel");
  if (rc) return rc;
  c->launches += 1;
  const double *alpha = kind == 1 ? ws : ns;
  const double *wsrc = kind == 1 ? mns : ns;
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
  a.out1_ld = d;
  if ((rc = c->launch(op, d, dw, a))) return rc;
  // cross pass: (K W_T)(c_S) and its alpha-gradient
  PairArgs b = a;
  b.ny = nf_t;
  b.y = ct;
  b.w = kind == 1 ? mnt : nt;
  b.out0 = ktt;
  b.out1 = gt;
  if ((rc = c->launch(op, d, dw, b))) return rc;
  // match = |T|^2 + w_S . K_SS W_S - 2 w_S . K_ST W_T (w_S = n_S for currents)
  if ((rc = c->cuda(dot_f64(st, alpha, kts, nf * dw, scal + 1, 0), "dot"))) return rc;
  if ((rc = c->cuda(dot_f64(st, alpha, ktt, nf * dw, scal + 2, 0), "dot"))) return rc;
  if ((rc = c->cuda(scalar_combine(st, match_dev, scal + 0, 1.0, scal + 1, 1.0, scal + 2, -2.0), "combine"))) return rc;
  c->launches += 3;
  if (!grad_dev) return GBK_OK;
  if (kind == 2) {
    GBK_MEASURE_DISPATCH(*this, measure_grad_kernel, nblk(nf), st, nf, exact, kts, ktt, gs, gt, sg, kt, gk);
    if ((rc = c->cuda(cudaGetLastError(), "measure_grad_kernel"))) return rc;
    GBK_MEASURE_DISPATCH(*this, measure_gather_kernel, nblk(nv), st, nv, pts_s, tris, csr_ptr, csr_fc, kt, gk,
                         grad_dev, scale, accumulate);
    c->launches += 2;
    return c->cuda(cudaGetLastError(), "measure_gather_kernel");
  }
  GBK_CELL_DISPATCH(*this, cell_grad_kernel, nblk(nf), st, nf, kind, ns, mns, kts, ktt, gs, gt, kt, gk);
  if ((rc = c->cuda(cudaGetLastError(), "cell_grad_kernel"))) return rc;
  GBK_CELL_DISPATCH(*this, vertex_gather_kernel, nblk(nv), st, nv, pts_s, tris, csr_ptr, csr_fc, kt, gk, grad_dev,
                    scale, accumulate);
  c->launches += 2;
  return c->cuda(cudaGetLastError(), "vertex_gather_kernel");
}

}  // namespace gbk

using namespace gbk;

static int surface_match(gbk_ctx *c, int kind, int d, int cell, long nv, const double *pts, long nf,
                         const int *tris, long nv_t, const double *pts_t, long nf_t, const int *tris_t,
                         double sigma, double *match, double *grad, const double *w = nullptr,
                         const double *w_t = nullptr) {
  if (!c) return GBK_ERR_ARG;
  c->err.clear();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (nv <= 0 || nf <= 0 || nv_t <= 0 || nf_t <= 0) return c->fail(GBK_ERR_ARG, "empty mesh");
  if (!pts || !pts_t || !match || (cell > 1 && (!tris || !tris_t))) return c->fail(GBK_ERR_ARG, "null pointer");
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "dimension %d not supported", d);
  if (c->capturing()) return c->fail(GBK_ERR_STATE, "the stand-alone data term allocates; use a registration object under capture");
  // cells are needed on the host for the vertex -> cell lists
  std::vector<int> th, tth;
  if (cell > 1) {
    th.resize((size_t)nf * cell);
    tth.resize((size_t)nf_t * cell);
    cudaMemcpy(th.data(), tris, th.size() * sizeof(int), cudaMemcpyDefault);
    cudaMemcpy(tth.data(), tris_t, tth.size() * sizeof(int), cudaMemcpyDefault);
    if (int rc = c->cuda(cudaGetLastError(), "copy cells")) return rc;
  }
  SurfaceTerm s;
  int rc = s.init(c, kind, d, cell, sigma, nv, nf, th.data(), nv_t, nf_t, tth.data(), w, w_t);
  if (!rc) {
    HostIO io(c);
    const double *dp = io.in(pts, (size_t)nv * d, "pts");
    const double *dpt = io.in(pts_t, (size_t)nv_t * d, "pts_t");
    double *dm = io.out(match, 1, "match");
    double *dg = io.out(grad, grad ? (size_t)nv * d : 0, "grad");
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
  return surface_match(c, 0, 3, 3, nv, pts, nf, tris, nv_t, pts_t, nf_t, tris_t, sigma, match, grad);
}

int gbk_varifold_match(gbk_ctx *c, long nv, const double *pts, long nf, const int *tris, long nv_t,
                       const double *pts_t, long nf_t, const int *tris_t, double sigma,
                       double *match, double *grad) {
  return surface_match(c, 1, 3, 3, nv, pts, nf, tris, nv_t, pts_t, nf_t, tris_t, sigma, match, grad);
}

int gbk_curve_currents_match(gbk_ctx *c, int d, long nv, const double *pts, long nseg, const int *segs, long nv_t,
                             const double *pts_t, long nseg_t, const int *segs_t, double sigma, double *match,
                             double *grad) {
  return surface_match(c, 0, d, 2, nv, pts, nseg, segs, nv_t, pts_t, nseg_t, segs_t, sigma, match, grad);
}

int gbk_curve_varifold_match(gbk_ctx *c, int d, long nv, const double *pts, long nseg, const int *segs, long nv_t,
                             const double *pts_t, long nseg_t, const int *segs_t, double sigma, double *match,
                             double *grad) {
  return surface_match(c, 1, d, 2, nv, pts, nseg, segs, nv_t, pts_t, nseg_t, segs_t, sigma, match, grad);
}

int gbk_pointcloud_match(gbk_ctx *c, int d, long n, const double *pts, const double *w, long n_t,
                         const double *pts_t, const double *w_t, double sigma, double *match, double *grad) {
  return surface_match(c, 2, d, 1, n, pts, n, nullptr, n_t, pts_t, n_t, nullptr, sigma, match, grad, w, w_t);
}

int gbk_volume_match(gbk_ctx *c, int d, long nv, const double *pts, long ncell, const int *cells, long nv_t,
                     const double *pts_t, long ncell_t, const int *cells_t, double sigma, double *match,
                     double *grad) {
  return surface_match(c, 2, d, d + 1, nv, pts, ncell, cells, nv_t, pts_t, ncell_t, cells_t, sigma, match, grad);
}

int gbk_landmark_match(gbk_ctx *c, int d, long n, const double *pts, const double *pts_t, double *match,
                       double *grad) {
  return surface_match(c, 3, d, 1, n, pts, n, nullptr, n, pts_t, n, nullptr, 1.0, match, grad);
}

}  // extern "C"
