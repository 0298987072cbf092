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
  pdl_entry();
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

// What a windowed image kernel accumulates per pixel p over the control points j whose window holds p:
//  IMG_CONV: V_p = sum_j W_j K_pj (ConvolveImageFast; D weight columns);
//  IMG_GRAD: G_p(k, l) = sum_j W_jk (x_p - y_j)_l (-2 K_pj / sigma^2) (ConvolveGradientImageFast(X, image));
//  IMG_GRAD_ALPHA: sum_k alpha_pk G_p(k, l) (ConvolveGradientImageFast(X, alpha, image)).
// The gradients take DV (1..3) weight columns at a time; wider weights run as column chunks.
enum { IMG_CONV = 0, IMG_GRAD = 1, IMG_GRAD_ALPHA = 2 };

struct ImageArgs {
  const double *x, *y, *w, *alpha;
  int w_ld, alpha_ld;  // leading dimensions of w and alpha (pointers already offset to the chunk)
  const int *start;
  long ny;
  double s2, pre;
  double *out;
  int out_ld;   // doubles per output row
  int acc_out;  // IMG_GRAD_ALPHA: add into out (later column chunks)
};

// F32 = false: FP64 as the reference (exp, no contracted multiply-adds, its order of operations).
// F32 = true (GBK_MODE_F32C): offsets from the tile's centre formed in FP64 and scaled by
// sqrt(log2 e) / sigma, then FP32 distances, K = 2^-r2 on the MUFU unit and per-pixel compensated
// FP32 sums (TwoSum), added up in FP64 at the end (the gradients' -2 / (sigma^2 pre) applied there).
template <int D, int DV, int KIND, bool F32>
__global__ void __launch_bounds__(kThreads) image_fast_kernel(const ImageArgs a, const ImageGeom g) {
  pdl_entry();
  typedef Tile<D> T;
  constexpr int NW = KIND == IMG_CONV ? D : DV;      // weight columns staged per control point
  constexpr int NA = KIND == IMG_CONV ? D : DV * D;  // accumulators per pixel
  __shared__ double s_y[F32 ? 1 : kThreads][D], s_w[F32 ? 1 : kThreads][NW];
  __shared__ float s_yf[F32 ? kThreads : 1][D], s_wf[F32 ? kThreads : 1][NW];
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
  const double s2 = a.s2, pre = a.pre;
  double xp[D], ctr[D], acc[NA];
  float xf[D], fs[NA], fc[NA];
  for (int k = 0; k < D; ++k) {
    xp[k] = valid ? a.x[row * D + k] : 0.0;
    ctr[k] = g.origin[k] + g.spacing[k] * 0.5 * (double)(lo[k] + hi[k] - 1);
    xf[k] = (float)((xp[k] - ctr[k]) * pre);
  }
  for (int m = 0; m < NA; ++m) {
    acc[m] = 0.0;
    fs[m] = 0.f;
    fc[m] = 0.f;
  }
  const int lane = tid & 31, warp = tid >> 5;
  for (long c0 = 0; c0 < a.ny; c0 += kThreads) {
    const long j = c0 + tid;
    int st[D];
    bool keep = j < a.ny;
    if (keep)
      for (int k = 0; k < D; ++k) {
        st[k] = a.start[j * D + k];
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
        if (F32)
          s_yf[pos][k] = (float)((a.y[j * D + k] - ctr[k]) * pre);
        else
          s_y[pos][k] = a.y[j * D + k];
        s_start[pos][k] = st[k];
      }
      for (int k = 0; k < NW; ++k) {
        if (F32)
          s_wf[pos][k] = (float)a.w[j * a.w_ld + k];
        else
          s_w[pos][k] = a.w[j * a.w_ld + k];
      }
    }
    __syncthreads();
    if (valid)
      for (int m = 0; m < total; ++m) {
        bool in = true;
        for (int k = 0; k < D; ++k) in = in && q[k] >= s_start[m][k] && q[k] < (long)s_start[m][k] + g.L;
        if (!in) continue;
        if (F32) {
          float r2 = 0.f, df[D];
          for (int k = 0; k < D; ++k) {
            df[k] = xf[k] - s_yf[m][k];
            r2 = fmaf(df[k], df[k], r2);
          }
          const float K = image_ex2(-r2);
          for (int c = 0; c < NA; ++c) {  // TwoSum into (fs, fc)
            const float v = KIND == IMG_CONV ? s_wf[m][c] * K : s_wf[m][c / D] * (K * df[c % D]);
            const float t = fs[c] + v, bp = t - fs[c];
            fc[c] += (fs[c] - (t - bp)) + (v - bp);
            fs[c] = t;
          }
        } else {
          double sq = 0.0, diff[D];
          for (int k = 0; k < D; ++k) {
            diff[k] = __dsub_rn(xp[k], s_y[m][k]);
            sq = __dadd_rn(sq, __dmul_rn(diff[k], diff[k]));
          }
          const double K = exp(-sq / s2);
          if (KIND == IMG_CONV) {
            for (int k = 0; k < D; ++k) acc[k] = __dadd_rn(acc[k], __dmul_rn(s_w[m][k], K));
          } else {  // ExactKernel::EvaluateKernelGradient: (x - y) * (-2 K / sigma^2)
            const double f = __ddiv_rn(__dmul_rn(-2.0, K), s2);
            for (int k = 0; k < DV; ++k)
              for (int l = 0; l < D; ++l)
                acc[k * D + l] = __dadd_rn(acc[k * D + l], __dmul_rn(__dmul_rn(diff[l], f), s_w[m][k]));
          }
        }
      }
    __syncthreads();
  }
  if (!valid) return;
  const double gs = -2.0 / (s2 * pre);  // F32 gradients were accumulated as K (x' - y')
  double v[NA];
  for (int c = 0; c < NA; ++c) v[c] = F32 ? (KIND == IMG_CONV ? 1.0 : gs) * ((double)fs[c] + (double)fc[c]) : acc[c];
  double *o = a.out + row * (long)a.out_ld;
  if (KIND == IMG_GRAD_ALPHA) {  // G_p^T alpha_p, summed over k in order
    for (int l = 0; l < D; ++l) {
      double s = 0.0;
      for (int k = 0; k < DV; ++k) s = __dadd_rn(s, __dmul_rn(v[k * D + l], a.alpha[row * a.alpha_ld + k]));
      o[l] = a.acc_out ? __dadd_rn(o[l], s) : s;
    }
  } else {
    for (int c = 0; c < NA; ++c) o[c] = v[c];
  }
}

template <int D>
__global__ void image_points_kernel(ImageGeom g, double *out) {
  pdl_entry();
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
  pdl_entry();
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double s = b ? __dadd_rn(a[i], b[i]) : a[i];
  out[i] = __dsub_rn(base[i], __dmul_rn(s, f));
}

// flag = 1 when a column of the n x D rows leaves [bbox[k][0], bbox[k][1]] (one CTA)
template <int D>
__global__ void out_of_box_kernel(const double *p, long n, const double *bbox, int *flag) {
  pdl_entry();
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

template <int D, int KIND, bool F32>
void launch_image_kind(int dv, unsigned nb, cudaStream_t st, const ImageArgs &a, const ImageGeom &g) {
  if (KIND == IMG_CONV || dv == 3)
    image_fast_kernel<D, 3, KIND, F32><<<nb, kThreads, 0, st>>>(a, g);
  else if (dv == 2)
    image_fast_kernel<D, 2, KIND, F32><<<nb, kThreads, 0, st>>>(a, g);
  else
    image_fast_kernel<D, 1, KIND, F32><<<nb, kThreads, 0, st>>>(a, g);
}

template <int KIND>
void launch_image_d(int d, bool f32, int dv, unsigned nb, cudaStream_t st, const ImageArgs &a, const ImageGeom &g) {
  if (d == 3) {
    if (f32)
      launch_image_kind<3, KIND, true>(dv, nb, st, a, g);
    else
      launch_image_kind<3, KIND, false>(dv, nb, st, a, g);
  } else {
    if (f32)
      launch_image_kind<2, KIND, true>(dv, nb, st, a, g);
    else
      launch_image_kind<2, KIND, false>(dv, nb, st, a, g);
  }
}

// One windowed pass of `kind` over the image; the gradients run the dv weight columns as chunks of at
// most 3 (IMG_GRAD writes its columns of each [p][k][l] row; IMG_GRAD_ALPHA adds the chunks up).
int launch_fast(gbk_ctx *c, const ImageGeom &g, int kind, const double *x, const double *y, const double *w, int dv,
                const double *alpha, const int *start, long ny, double sigma, double *out) {
  const long tiles = g.d == 3 ? ((g.n[0] + 7) / 8) * ((g.n[1] + 7) / 8) * ((g.n[2] + 3) / 4)
                              : ((g.n[0] + 15) / 16) * ((g.n[1] + 15) / 16);
  if (tiles > 2147483647L) return c->fail(GBK_ERR_ARG, "image too large");
  const bool f32 = c->mode != GBK_MODE_F64;
  const unsigned nb = (unsigned)tiles;
  ImageArgs a;
  a.x = x;
  a.y = y;
  a.start = start;
  a.ny = ny;
  a.s2 = sigma * sigma;
  a.pre = std::sqrt(1.4426950408889634) / sigma;  // sqrt(log2 e) / sigma
  a.w_ld = dv;
  a.alpha_ld = dv;
  if (kind == IMG_CONV) {
    a.w = w;
    a.alpha = nullptr;
    a.out = out;
    a.out_ld = g.d;
    a.acc_out = 0;
    launch_image_d<IMG_CONV>(g.d, f32, g.d, nb, c->stream, a, g);
    c->launches += 1;
    return c->cuda(cudaGetLastError(), "image convolution");
  }
  for (int c0 = 0; c0 < dv; c0 += 3) {
    const int cw = std::min(3, dv - c0);
    a.w = w + c0;
    a.alpha = alpha ? alpha + c0 : nullptr;
    a.acc_out = c0 > 0;
    if (kind == IMG_GRAD) {
      a.out = out + (long)c0 * g.d;
      a.out_ld = dv * g.d;
      launch_image_d<IMG_GRAD>(g.d, f32, cw, nb, c->stream, a, g);
    } else {
      a.out = out;
      a.out_ld = g.d;
      launch_image_d<IMG_GRAD_ALPHA>(g.d, f32, cw, nb, c->stream, a, g);
    }
    c->launches += 1;
    if (int rc = c->cuda(cudaGetLastError(), "image gradient")) return rc;
  }
  return GBK_OK;
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
  if (int rc = launch_fast(c, g, IMG_CONV, dx, dy, dw, d, nullptr, start, ny, sigma, dout)) return rc;
  return io.finish();
}

// ExactKernel::ConvolveGradientImageFast, both overloads: alpha == null gives the gradients
// (nx x dv x d), else their contraction with alpha (nx x d).
static int image_gradient(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y, const double *w,
                          long ny, double sigma, const double *alpha, const double *origin, const double *spacing,
                          const long *size, double *out) {
  if (sigma < 1e-10) sigma = 1e-10;  // AbstractKernel::SetKernelWidth
  ImageGeom g;
  if (int rc = geom_from(c, d, origin, spacing, size, sigma, &g)) return rc;
  if (nx != g.pixels()) return c->fail(GBK_ERR_ARG, "x has %ld rows for an image of %ld pixels", nx, g.pixels());
  if (ny <= 0) return c->fail(GBK_ERR_ARG, "need at least one control point");
  if (dv <= 0) return c->fail(GBK_ERR_ARG, "weights need at least one column (dv=%d)", dv);
  if (!x || !y || !w || !out) return c->fail(GBK_ERR_ARG, "null pointer");
  if (c->capturing()) return c->fail(GBK_ERR_STATE, "reads back the window check; not under stream capture");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  const double *da = alpha ? io.in(alpha, (size_t)nx * dv, "alpha") : nullptr;
  double *dout = io.out(out, (size_t)nx * (alpha ? d : dv * d), "out");
  if (io.rc) return io.rc;
  const size_t b_start = up256((size_t)ny * d * sizeof(int));
  if (int rc = c->ensure(c->tmp, b_start + 256, "image windows")) return rc;
  int *start = (int *)c->tmp.p;
  int *bad = (int *)((char *)c->tmp.p + b_start);
  std::vector<int> bad_host;
  if (int rc = windows(c, g, dy, ny, 1, sigma, start, bad, bad_host)) return rc;
  if (bad_host[0] != 0x7f7f7f7f)
    return c->fail(GBK_ERR_ARG, "control point %d: its window misses the image", bad_host[0]);
  if (int rc = launch_fast(c, g, alpha ? IMG_GRAD_ALPHA : IMG_GRAD, dx, dy, dw, dv, da, start, ny, sigma, dout))
    return rc;
  return io.finish();
}

int gbk_convolve_gradient_image_fast(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y,
                                     const double *w, long ny, double sigma, const double *origin,
                                     const double *spacing, const long *size, double *out) {
  GBK_IMAGE_GUARD(c);
  GBK_RANGE();
  return image_gradient(c, d, dv, x, nx, y, w, ny, sigma, nullptr, origin, spacing, size, out);
}

int gbk_convolve_gradient_image_fast_alpha(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y,
                                           const double *w, long ny, double sigma, const double *alpha,
                                           const double *origin, const double *spacing, const long *size,
                                           double *out) {
  GBK_IMAGE_GUARD(c);
  GBK_RANGE();
  if (!alpha) return c->fail(GBK_ERR_ARG, "null pointer");
  return image_gradient(c, d, dv, x, nx, y, w, ny, sigma, alpha, origin, spacing, size, out);
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
      return launch_fast(c, g, IMG_CONV, X, dpos + (size_t)t * n, dmom + (size_t)t * n, d, nullptr,
                         start + (size_t)t * n, ncp, sigma, V);
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
