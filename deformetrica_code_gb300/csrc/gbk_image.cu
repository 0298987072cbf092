// The image-grid side of the kernel path on the device.
//
// gbk_convolve_image_fast restates ExactKernel::ConvolveImageFast
// (src/support/kernels/ExactKernel.cxx:76-129): every control point y_j adds W_j K(X_p, y_j) to the
// pixels p of a window of int(6 sigma) pixels per axis that starts at the index of y_j - 3 sigma
// (ITK's TransformPhysicalPointToIndex, rounded half up) and is cropped to the image; X holds one
// (deformed) point per pixel, first index fastest (GridFunctions::ImageToPoints). The reference
// loops over control points and scatters; here each CTA owns a tile of pixels, keeps the control
// points whose window meets the tile (in control-point order, compacted through shared memory) and
// each thread gathers its pixel's sum in that order, so every pixel sees the reference's order of
// additions. GBK_MODE_F64 evaluates in FP64 without contracted multiply-adds, as the reference's
// scalar loop; GBK_MODE_F32C evaluates the exponentials in FP32 with compensated per-pixel sums.
//
// gbk_flow_image_maps restates the backward integration of the image maps
// (src/core/model_tools/deformations/Diffeos.cxx:725-770, non-regression branch) with either the
// windowed sum or the full kernel sum (the context's precision), Euler or Heun, and the bounding-box
// stop of Diffeos::CheckBoundingBox (:187-198).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_hostio.h"
#include "gbk_ops.h"

using namespace gbk;

namespace {

constexpr int kThreads = 256;

struct ImageGeom {
  int d;
  long n[3];
  double origin[3], spacing[3];
  int L;  // window size in pixels per axis
  __host__ __device__ long pixels() const { return n[0] * n[1] * (d == 3 ? n[2] : 1); }
};

template <int D>
struct Tile;
template <>
struct Tile<2> {
  static constexpr int X = 16, Y = 16, Z = 1;
};
template <>
struct Tile<3> {
  static constexpr int X = 8, Y = 8, Z = 4;
};

unsigned blocks_for(long n, int bs = kThreads) { return (unsigned)std::max(1L, (n + bs - 1) / bs); }

// window start indices of n control points (rows of y) and, per group of `per` rows, the first row
// whose window misses the image (or INT_MAX)
template <int D>
__global__ void image_windows_kernel(const double *y, long n, long per, double sigma, ImageGeom g, int *start,
                                     int *bad) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  bool ok = g.L > 0;
  for (int k = 0; k < D; ++k) {
    const double p = __dsub_rn(y[r * D + k], __dmul_rn(3.0, sigma));  // rounded as y - 3 sigma is
    double v = floor((p - g.origin[k]) / g.spacing[k] + 0.5);
    v = fmin(fmax(v, -1073741824.0), 1073741824.0);
    const int s = (int)v;
    start[r * D + k] = s;
    ok = ok && (long)s < g.n[k] && (long)s + g.L > 0;
  }
  if (!ok) atomicMin(bad + r / per, (int)(r % per));
}

__device__ __forceinline__ float image_ex2(float v) {
  float r;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}

// F32 = false: FP64 as the reference (exp, no contracted multiply-adds). F32 = true (GBK_MODE_F32C):
// offsets from the tile's centre formed in FP64 and scaled by sqrt(log2 e) / sigma, then FP32 distances,
// K = 2^-r2 on the MUFU unit and per-pixel compensated FP32 sums (TwoSum), added up in FP64 at the end.
template <int D, bool F32>
__global__ void __launch_bounds__(kThreads) image_fast_kernel(const double *x, const double *y, const double *w,
                                                              const int *start, long ny, double s2, double pre,
                                                              ImageGeom g, double *out) {
  typedef Tile<D> T;
  __shared__ double s_y[F32 ? 1 : kThreads][D], s_w[F32 ? 1 : kThreads][D];
  __shared__ float s_yf[F32 ? kThreads : 1][D], s_wf[F32 ? kThreads : 1][D];
  __shared__ int s_start[kThreads][D];
  __shared__ int s_warp[kThreads / 32 + 1];
  const int tid = threadIdx.x;
  const long tiles0 = (g.n[0] + T::X - 1) / T::X, tiles1 = (g.n[1] + T::Y - 1) / T::Y;
  const long b = blockIdx.x;
  long lo[3] = {(b % tiles0) * T::X, ((b / tiles0) % tiles1) * T::Y, D == 3 ? (b / (tiles0 * tiles1)) * T::Z : 0};
  long hi[3] = {lo[0] + T::X < g.n[0] ? lo[0] + T::X : g.n[0], lo[1] + T::Y < g.n[1] ? lo[1] + T::Y : g.n[1],
                D == 3 ? (lo[2] + T::Z < g.n[2] ? lo[2] + T::Z : g.n[2]) : 1};
  const long q[3] = {lo[0] + tid % T::X, lo[1] + (tid / T::X) % T::Y, lo[2] + tid / (T::X * T::Y)};
  const bool valid = q[0] < hi[0] && q[1] < hi[1] && (D == 2 || q[2] < hi[2]);
  const long row = q[0] + g.n[0] * (q[1] + (D == 3 ? g.n[1] * q[2] : 0));
  double xp[D], acc[D], ctr[D];
  float xf[D], fs[D], fc[D];
  for (int k = 0; k < D; ++k) {
    xp[k] = valid ? x[row * D + k] : 0.0;
    acc[k] = 0.0;
    ctr[k] = g.origin[k] + g.spacing[k] * 0.5 * (double)(lo[k] + hi[k] - 1);
    xf[k] = (float)((xp[k] - ctr[k]) * pre);
    fs[k] = 0.f;
    fc[k] = 0.f;
  }
  const int lane = tid & 31, warp = tid >> 5;
  for (long c0 = 0; c0 < ny; c0 += kThreads) {
    const long j = c0 + tid;
    int st[D];
    bool keep = j < ny;
    if (keep)
      for (int k = 0; k < D; ++k) {
        st[k] = start[j * D + k];
        keep = keep && (long)st[k] < hi[k] && (long)st[k] + g.L > lo[k];
      }
    // order-preserving compaction of the kept control points
    const unsigned ball = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) s_warp[warp] = __popc(ball);
    __syncthreads();
    int base = 0, total = 0;
    for (int v = 0; v < kThreads / 32; ++v) {
      base += v < warp ? s_warp[v] : 0;
      total += s_warp[v];
    }
    if (keep) {
      const int pos = base + __popc(ball & ((1u << lane) - 1u));
      for (int k = 0; k < D; ++k) {
        if (F32) {
          s_yf[pos][k] = (float)((y[j * D + k] - ctr[k]) * pre);
          s_wf[pos][k] = (float)w[j * D + k];
        } else {
          s_y[pos][k] = y[j * D + k];
          s_w[pos][k] = w[j * D + k];
        }
        s_start[pos][k] = st[k];
      }
    }
    __syncthreads();
    if (valid)
      for (int m = 0; m < total; ++m) {
        bool in = true;
        for (int k = 0; k < D; ++k) in = in && q[k] >= s_start[m][k] && q[k] < (long)s_start[m][k] + g.L;
        if (!in) continue;
        if (F32) {
          float r2 = 0.f;
          for (int k = 0; k < D; ++k) {
            const float df = xf[k] - s_yf[m][k];
            r2 = fmaf(df, df, r2);
          }
          const float K = image_ex2(-r2);
          for (int k = 0; k < D; ++k) {  // TwoSum into (fs, fc)
            const float v = s_wf[m][k] * K;
            const float t = fs[k] + v, bp = t - fs[k];
            fc[k] += (fs[k] - (t - bp)) + (v - bp);
            fs[k] = t;
          }
        } else {
          double sq = 0.0;
          for (int k = 0; k < D; ++k) {
            const double diff = __dsub_rn(xp[k], s_y[m][k]);
            sq = __dadd_rn(sq, __dmul_rn(diff, diff));
          }
          const double K = exp(-sq / s2);
          for (int k = 0; k < D; ++k) acc[k] = __dadd_rn(acc[k], __dmul_rn(s_w[m][k], K));
        }
      }
    __syncthreads();
  }
  if (valid)
    for (int k = 0; k < D; ++k) out[row * D + k] = F32 ? (double)fs[k] + (double)fc[k] : acc[k];
}

template <int D>
__global__ void image_points_kernel(ImageGeom g, double *out) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= g.pixels()) return;
  long rem = r;
  for (int k = 0; k < D; ++k) {
    const long q = rem % g.n[k];
    rem /= g.n[k];
    out[r * D + k] = __dadd_rn(g.origin[k], __dmul_rn(g.spacing[k], (double)q));  // no contraction, as ITK
  }
}

// out = base - dt a (Euler), or base - (a + b) h (Heun), rounded as written
__global__ void back_step_kernel(double *out, const double *base, const double *a, const double *b, double f, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = b ? __dadd_rn(a[i], b[i]) : a[i];
  out[i] = __dsub_rn(base[i], __dmul_rn(s, f));
}

// flag = 1 when a column of the n x D rows leaves [bbox[k][0], bbox[k][1]] (one CTA)
template <int D>
__global__ void out_of_box_kernel(const double *p, long n, const double *bbox, int *flag) {
  __shared__ int s_out;
  if (threadIdx.x == 0) s_out = 0;
  __syncthreads();
  int out = 0;
  for (long i = threadIdx.x; i < n; i += blockDim.x)
    for (int k = 0; k < D; ++k) {
      const double v = p[i * D + k];
      out |= (v < bbox[2 * k] || v > bbox[2 * k + 1]) ? 1 : 0;
    }
  if (out) atomicOr(&s_out, 1);
  __syncthreads();
  if (threadIdx.x == 0) *flag = s_out;
}

int geom_from(gbk_ctx *c, int d, const double *origin, const double *spacing, const long *size, double sigma,
              ImageGeom *g) {
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "dimension %d not supported", d);
  if (!origin || !spacing || !size) return c->fail(GBK_ERR_ARG, "null image geometry");
  g->d = d;
  for (int k = 0; k < 3; ++k) {
    g->n[k] = k < d ? size[k] : 1;
    g->origin[k] = k < d ? origin[k] : 0.0;
    g->spacing[k] = k < d ? spacing[k] : 1.0;
    if (g->n[k] <= 0 || g->n[k] > (1L << 30)) return c->fail(GBK_ERR_ARG, "image size out of range");
    if (!(g->spacing[k] > 0)) return c->fail(GBK_ERR_ARG, "image spacing must be positive");
  }
  if (g->pixels() > (1L << 31)) return c->fail(GBK_ERR_ARG, "image of more than 2^31 pixels");
  const double L = 6 * sigma;
  if (!(L >= 1.0)) return c->fail(GBK_ERR_ARG, "window int(6 sigma) = 0 pixels (sigma %g)", sigma);
  g->L = L > 1073741824.0 ? 1073741824 : (int)L;
  return GBK_OK;
}

// Window starts of `groups` x `per` control points (rows of y) into `start`; bad_host[g] = the first
// control point of group g whose window misses the image, or 0x7f7f7f7f when none does (the
// caller turns a miss into GBK_ERR_ARG when it needs that group). Waits for the stream.
int windows(gbk_ctx *c, const ImageGeom &g, const double *y, long per, int groups, double sigma, int *start,
            int *bad_dev, std::vector<int> &bad_host) {
  cudaStream_t st = c->stream;
  int rc = c->cuda(cudaMemsetAsync(bad_dev, 0x7f, groups * sizeof(int), st), "memset");
  if (rc) return rc;
  const long n = per * groups;
  if (g.d == 3)
    image_windows_kernel<3><<<blocks_for(n), kThreads, 0, st>>>(y, n, per, sigma, g, start, bad_dev);
  else
    image_windows_kernel<2><<<blocks_for(n), kThreads, 0, st>>>(y, n, per, sigma, g, start, bad_dev);
  c->launches += 1;
  if ((rc = c->cuda(cudaGetLastError(), "image windows"))) return rc;
  bad_host.assign(groups, 0);
  rc = c->cuda(cudaMemcpyAsync(bad_host.data(), bad_dev, groups * sizeof(int), cudaMemcpyDeviceToHost, st), "D2H");
  if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
  return rc;
}

int launch_fast(gbk_ctx *c, const ImageGeom &g, const double *x, const double *y, const double *w, const int *start,
                long ny, double sigma, double *out) {
  const long tiles = g.d == 3 ? ((g.n[0] + 7) / 8) * ((g.n[1] + 7) / 8) * ((g.n[2] + 3) / 4)
                              : ((g.n[0] + 15) / 16) * ((g.n[1] + 15) / 16);
  if (tiles > 2147483647L) return c->fail(GBK_ERR_ARG, "image too large");
  const double s2 = sigma * sigma, pre = std::sqrt(1.4426950408889634) / sigma;  // sqrt(log2 e) / sigma
  const bool f32 = c->mode != GBK_MODE_F64;
  const unsigned nb = (unsigned)tiles;
  if (g.d == 3) {
    if (f32)
      image_fast_kernel<3, true><<<nb, kThreads, 0, c->stream>>>(x, y, w, start, ny, s2, pre, g, out);
    else
      image_fast_kernel<3, false><<<nb, kThreads, 0, c->stream>>>(x, y, w, start, ny, s2, pre, g, out);
  } else {
    if (f32)
      image_fast_kernel<2, true><<<nb, kThreads, 0, c->stream>>>(x, y, w, start, ny, s2, pre, g, out);
    else
      image_fast_kernel<2, false><<<nb, kThreads, 0, c->stream>>>(x, y, w, start, ny, s2, pre, g, out);
  }
  c->launches += 1;
  return c->cuda(cudaGetLastError(), "image convolution");
}

size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

#define GBK_IMAGE_GUARD(ctx)                                                 \
  do {                                                                       \
    if (!(ctx)) return GBK_ERR_ARG;                                          \
    (ctx)->err.clear();                                                      \
    if (cudaSetDevice((ctx)->device) != cudaSuccess) {                       \
      cudaGetLastError();                                                    \
      return (ctx)->fail(GBK_ERR_CUDA, "cudaSetDevice(%d)", (ctx)->device);  \
    }                                                                        \
  } while (0)

extern "C" {

int gbk_image_points(gbk_ctx *c, int d, const double *origin, const double *spacing, const long *size,
                     double *points) {
  GBK_IMAGE_GUARD(c);
  GBK_RANGE();
  ImageGeom g;
  if (int rc = geom_from(c, d, origin, spacing, size, 1.0, &g)) return rc;
  if (!points) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  double *dp = io.out(points, (size_t)g.pixels() * d, "points");
  if (io.rc) return io.rc;
  if (d == 3)
    image_points_kernel<3><<<blocks_for(g.pixels()), kThreads, 0, c->stream>>>(g, dp);
  else
    image_points_kernel<2><<<blocks_for(g.pixels()), kThreads, 0, c->stream>>>(g, dp);
  c->launches += 1;
  if (int rc = c->cuda(cudaGetLastError(), "image points")) return rc;
  return io.finish();
}

int gbk_convolve_image_fast(gbk_ctx *c, int d, const double *x, long nx, const double *y, const double *w, long ny,
                            double sigma, const double *origin, const double *spacing, const long *size,
                            double *out) {
  GBK_IMAGE_GUARD(c);
  GBK_RANGE();
  if (sigma < 1e-10) sigma = 1e-10;  // AbstractKernel::SetKernelWidth
  ImageGeom g;
  if (int rc = geom_from(c, d, origin, spacing, size, sigma, &g)) return rc;
  if (nx != g.pixels()) return c->fail(GBK_ERR_ARG, "x has %ld rows for an image of %ld pixels", nx, g.pixels());
  if (ny <= 0) return c->fail(GBK_ERR_ARG, "need at least one control point");
  if (!x || !y || !w || !out) return c->fail(GBK_ERR_ARG, "null pointer");
  if (c->capturing()) return c->fail(GBK_ERR_STATE, "reads back the window check; not under stream capture");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * d, "w");
  double *dout = io.out(out, (size_t)nx * d, "out");
  if (io.rc) return io.rc;
  const size_t b_start = up256((size_t)ny * d * sizeof(int));
  if (int rc = c->ensure(c->tmp, b_start + 256, "image windows")) return rc;
  int *start = (int *)c->tmp.p;
  int *bad = (int *)((char *)c->tmp.p + b_start);
  std::vector<int> bad_host;
  if (int rc = windows(c, g, dy, ny, 1, sigma, start, bad, bad_host)) return rc;
  if (bad_host[0] != 0x7f7f7f7f)
    return c->fail(GBK_ERR_ARG, "control point %d: its window misses the image", bad_host[0]);
  if (int rc = launch_fast(c, g, dx, dy, dw, start, ny, sigma, dout)) return rc;
  return io.finish();
}

int gbk_flow_image_maps(gbk_ctx *c, int d, long ncp, const double *pos_traj, const double *mom_traj, int T,
                        double sigma, double span, int heun, int fast, const double *origin, const double *spacing,
                        const long *size, const double *bbox, double *maps_traj, int *stopped_at) {
  GBK_IMAGE_GUARD(c);
  GBK_RANGE();
  if (sigma < 1e-10) sigma = 1e-10;
  if (stopped_at) *stopped_at = -1;
  ImageGeom g;
  if (int rc = geom_from(c, d, origin, spacing, size, fast ? sigma : 1.0, &g)) return rc;
  if (ncp <= 0) return c->fail(GBK_ERR_ARG, "need at least one control point");
  if (T < 2) return c->fail(GBK_ERR_ARG, "need at least two time points (T=%d)", T);
  if (!pos_traj || !mom_traj || !maps_traj) return c->fail(GBK_ERR_ARG, "null pointer");
  if (c->capturing()) return c->fail(GBK_ERR_STATE, "reads back the checks of every step; not under stream capture");
  const long npix = g.pixels(), m = npix * d, n = ncp * d;
  cudaStream_t st = c->stream;
  HostIO io(c);
  const double *dpos = io.in(pos_traj, (size_t)T * n, "pos_traj");
  const double *dmom = io.in(mom_traj, (size_t)T * n, "mom_traj");
  double *dmaps = io.out(maps_traj, (size_t)T * m, "maps_traj");
  if (io.rc) return io.rc;
  // scratch: dY, dY2, window starts of every time point, per-time window verdicts, the box and flags
  const size_t b_v = up256((size_t)m * sizeof(double)), b_start = up256((size_t)T * n * sizeof(int));
  const size_t b_bad = up256((size_t)T * sizeof(int));
  if (int rc = c->ensure(c->tmp, 2 * b_v + b_start + b_bad + 512, "image flow scratch")) return rc;
  char *base = (char *)c->tmp.p;
  double *dY = (double *)base, *dY2 = (double *)(base + b_v);
  int *start = (int *)(base + 2 * b_v);
  int *bad = (int *)(base + 2 * b_v + b_start);
  double *dbox = (double *)(base + 2 * b_v + b_start + b_bad);
  int *flag = (int *)(base + 2 * b_v + b_start + b_bad + 256);
  int rc;
  // every map starts as the image points
  if (d == 3)
    image_points_kernel<3><<<blocks_for(npix), kThreads, 0, st>>>(g, dmaps);
  else
    image_points_kernel<2><<<blocks_for(npix), kThreads, 0, st>>>(g, dmaps);
  c->launches += 1;
  if ((rc = c->cuda(cudaGetLastError(), "image points"))) return rc;
  for (int t = 1; t < T && !rc; ++t)
    rc = c->cuda(cudaMemcpyAsync(dmaps + (size_t)t * m, dmaps, m * sizeof(double), cudaMemcpyDeviceToDevice, st),
                 "copy");
  if (rc) return rc;
  // nearly zero initial momenta: no motion
  int small = 0;
  if ((rc = c->cuda(small_norm_flag(st, dmom, n, 1e-20, flag), "norm flag"))) return rc;
  c->launches += 1;
  if ((rc = c->cuda(cudaMemcpyAsync(&small, flag, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H"))) return rc;
  if ((rc = c->cuda(cudaStreamSynchronize(st), "sync"))) return rc;
  if (small) return io.finish();
  std::vector<int> bad_host;
  if (fast && (rc = windows(c, g, dpos, ncp, T, sigma, start, bad, bad_host))) return rc;
  if (bbox && (rc = c->cuda(cudaMemcpyAsync(dbox, bbox, 2 * d * sizeof(double), cudaMemcpyHostToDevice, st), "H2D")))
    return rc;
  const double dt = span / (T - 1);
  auto conv = [&](const double *X, int t, double *V) -> int {
    if (fast) {
      if (bad_host[t] != 0x7f7f7f7f)
        return c->fail(GBK_ERR_ARG, "time %d, control point %d: its window misses the image", t, bad_host[t]);
      return launch_fast(c, g, X, dpos + (size_t)t * n, dmom + (size_t)t * n, start + (size_t)t * n, ncp, sigma, V);
    }
    PairArgs a = pair_args(npix, ncp, sigma);
    a.x = X;
    a.y = dpos + (size_t)t * n;
    a.w = dmom + (size_t)t * n;
    a.w_ld = d;
    a.out0 = V;
    a.out0_ld = d;
    return c->launch(OP_CONV, d, d, a);
  };
  for (int t = T - 1; t >= 1; --t) {
    double *mt = dmaps + (size_t)t * m, *mt1 = dmaps + (size_t)(t - 1) * m;
    if ((rc = conv(mt, t, dY))) return rc;
    back_step_kernel<<<blocks_for(m), kThreads, 0, st>>>(mt1, mt, dY, nullptr, dt, m);
    c->launches += 1;
    if ((rc = c->cuda(cudaGetLastError(), "euler"))) return rc;
    if (heun) {
      if ((rc = conv(mt1, t - 1, dY2))) return rc;
      back_step_kernel<<<blocks_for(m), kThreads, 0, st>>>(mt1, mt, dY, dY2, dt * 0.5, m);
      c->launches += 1;
      if ((rc = c->cuda(cudaGetLastError(), "heun"))) return rc;
    }
    if (bbox) {
      if (d == 3)
        out_of_box_kernel<3><<<1, 1024, 0, st>>>(mt1, npix, dbox, flag);
      else
        out_of_box_kernel<2><<<1, 1024, 0, st>>>(mt1, npix, dbox, flag);
      c->launches += 1;
      int out = 0;
      if ((rc = c->cuda(cudaMemcpyAsync(&out, flag, sizeof(int), cudaMemcpyDeviceToHost, st), "D2H"))) return rc;
      if ((rc = c->cuda(cudaStreamSynchronize(st), "sync"))) return rc;
      if (out) {
        if (stopped_at) *stopped_at = t - 1;
        break;
      }
    }
  }
  return io.finish();
}

}  // extern "C"
