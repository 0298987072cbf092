// Particle-mesh Gaussian kernel sums on the device: the reference's P3MKernel
// (src/support/kernels/P3MKernel.cxx) with cuFFT. Steps, as the reference:
//   grid (DetermineGrids, :371-432): spacing ratio x sigma; per dimension the padded domain length
//     divided by the spacing, truncated and rounded up to a power of two; origin centring the grid;
//   splat (UpdateGrids, :237-347): multilinear weights to the 2^d grid points around each source,
//     points outside the grid, zero weights and "border" points (an index <= 0) left out;
//   kernel spectra (BuildFFTKernel / BuildFFTGradientKernels, :666-944): the Gaussian and its
//     gradient at the non-border grid points around the grid centre, inverse-FFT-shifted, FFT;
//   convolution (ApplyKernelFFT, :1088-1178): inverse FFT of the product of the spectra;
//   interpolation (Interpolate, :641-662): multilinear at the targets.
// Coordinates, interpolation weights and outputs are FP64; the grids, spectra and transforms are
// FP64 in GBK_MODE_F64 and FP32 in GBK_MODE_F32C (FP64 transforms are bound by the FP64 pipe, which
// is a small fraction of the FP32 one; FP32 grids add ~1e-6 relative to a method whose own error
// against the exact sum is ~1e-2). The splat accumulates with atomic adds (grid sums in arbitrary
// order, last-bit differences between runs). Each call runs one batched forward transform over
// the weight grids and one batched inverse transform over the images; plans, kernel spectra and
// scratch are cached in the context per grid, width and precision.
#include <cuda_runtime.h>
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_hostio.h"

namespace {

struct P3MGrid {
  int d = 3;
  long n[3] = {1, 1, 1};
  double origin[3] = {0, 0, 0};
  double s = 1.0;
  double inv_s = 1.0;  // 1 / s (FP32 grids: continuous indices by multiplication)
  long cells() const { return n[0] * n[1] * (d == 3 ? n[2] : 1); }
  long ccells() const { return n[0] * (d == 3 ? n[1] * (n[2] / 2 + 1) : (n[1] / 2 + 1)); }
};

struct P3MPlan {
  cufftType type;
  int batch;
  cufftHandle h;
};

struct P3MCache {
  bool valid = false;  // kspec holds the spectra of (d, n, s, sigma, f64)
  int d = 0;
  long n[3] = {0, 0, 0};
  double s = 0, sigma = 0;
  bool f64 = true;
  std::vector<P3MPlan> plans;  // for the grid n of d
  void *kspec = nullptr;       // kernel spectra: Gaussian, its d gradient components, its d(d+1)/2 Hessian entries
  void *work = nullptr;        // grow-only scratch: grids, images, spectra, products, box
  size_t work_bytes = 0;

  void drop_plans() {
    for (auto &p : plans) cufftDestroy(p.h);
    plans.clear();
  }
};

void p3m_cache_free(void *p) {
  P3MCache *c = (P3MCache *)p;
  if (!c) return;
  c->drop_plans();
  if (c->kspec) cudaFree(c->kspec);
  if (c->work) cudaFree(c->work);
  delete c;
}

// grows the cached scratch to at least `bytes` (contents not kept)
int p3m_work(gbk_ctx *c, P3MCache *pc, size_t bytes) {
  if (pc->work_bytes >= bytes) return 0;
  if (c->alloc_limit && bytes > c->alloc_limit)
    return c->fail(GBK_ERR_ALLOC, "P3M scratch: %zu bytes refused (injected allocation limit)", bytes);
  if (pc->work) {
    cudaStreamSynchronize(c->stream);
    cudaFree(pc->work);
  }
  pc->work = nullptr;
  pc->work_bytes = 0;
  int rc = c->cuda(cudaMalloc(&pc->work, bytes), "cudaMalloc (P3M)");
  if (!rc) pc->work_bytes = bytes;
  return rc;
}

unsigned nblk(long n, int bs = 256) { return (unsigned)std::max(1L, (n + bs - 1) / bs); }

// kernel images per grid: the Gaussian, its d gradient components, its d(d+1)/2 Hessian entries
// (r <= c, first row first: the reference's BuildFFTHessianKernels order)
inline int p3m_kernels(int d) { return 1 + d + d * (d + 1) / 2; }

// Kernel images in inverse-FFT-shifted layout: slot j holds the value at grid index (j + n/2) mod n.
template <int D, typename G>
__global__ void p3m_kernel_images(P3MGrid g, double sigma, G *img, long cells) {
  gbk::pdl_entry();
  long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cells) return;
  long slot[3], ind[3];
  long r = j;
  for (int k = D - 1; k >= 0; --k) {
    slot[k] = r % g.n[k];
    r /= g.n[k];
  }
  bool border = false;
  double d2 = 0.0, diff[3];
  for (int k = 0; k < D; ++k) {
    ind[k] = (slot[k] + g.n[k] / 2) % g.n[k];
    border = border || ind[k] <= 0;
    const double x = g.origin[k] + ind[k] * g.s;
    const double c = g.origin[k] + 0.5 * g.n[k] * g.s;
    diff[k] = x - c;
    d2 += diff[k] * diff[k];
  }
  const double s2 = sigma * sigma, kv = exp(-d2 / s2);
  img[j] = (G)(border ? 0.0 : kv);
  for (int k = 0; k < D; ++k) img[(1 + k) * cells + j] = (G)(border ? 0.0 : diff[k] * (-2.0 * kv / s2));
  // ExactKernel::EvaluateKernelHessian (ExactKernel.h:113-132): (x - c)(x - c)^T 4K/s^4 - 2K/s^2 I
  int q = 1 + D;
  for (int r = 0; r < D; ++r)
    for (int cc = r; cc < D; ++cc, ++q) {
      double h = diff[r] * diff[cc] * (4.0 * kv / (s2 * s2));
      if (r == cc) h -= 2.0 * kv / s2;
      img[(long)q * cells + j] = (G)(border ? 0.0 : h);
    }
}

// multilinear corners of one point, slot b = corner b in the reference's order (first dimension
// slowest): linear index, weight, `use` (inside the grid and weight > 0) and `interior` (no index
// <= 0, the splat's border rule). Fixed slots keep the arrays in registers. The continuous index
// (p - origin) / s is formed in FP64 (the reference's division on FP64 grids, a multiplication by
// the reciprocal spacing on FP32 grids); the fractions and weights are in the grid's precision G,
// so FP32 grids weigh and sum in FP32: GB300's FP64 rate is ~1/64 of its FP32 rate, and FP64
// weights and sums dominated these kernels while the FP32 grid values carry ~1e-7 relative anyway.
template <int D, typename G>
struct P3MCorners {
  long l[1 << D];
  G w[1 << D];
  bool use[1 << D], interior[1 << D];
};

template <int D, typename G>
__device__ inline void p3m_corners(const double *p, const P3MGrid &g, P3MCorners<D, G> &cs) {
  long i1[D];
  G f[D], h[D];
#pragma unroll
  for (int k = 0; k < D; ++k) {
    double c;
    if constexpr (std::is_same<G, double>::value)
      c = (p[k] - g.origin[k]) / g.s;
    else
      c = (p[k] - g.origin[k]) * g.inv_s;
    const double fl = floor(c);
    i1[k] = (long)fl;
    f[k] = (G)(c - fl);
    h[k] = (G)((fl + 1.0) - c);
  }
#pragma unroll
  for (int b = 0; b < (1 << D); ++b) {
    G wt = (G)1;
    bool in = true, inner = true;
    long l = 0;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const int bit = (b >> (D - 1 - k)) & 1;
      const long q = i1[k] + bit;
      wt *= bit ? f[k] : h[k];
      in = in && q >= 0 && q < g.n[k];
      inner = inner && q > 0;
      l = l * g.n[k] + q;
    }
    cs.l[b] = l;
    cs.w[b] = wt;
    cs.use[b] = in && wt > (G)0;
    cs.interior[b] = inner;
  }
}

// Splat into interleaved weight grids (cell-major, dvp slots per cell): FP32 grids add a source's
// weights into a corner's cell with one vector atomic per 4 slots (2 for two weights), FP64 grids
// with one atomic per weight. Padded slots receive zeros.
template <int D, typename G>
__global__ void p3m_splat(const double *y, const double *wts, long ny, int dv, int dvp, P3MGrid g, G *grids) {
  gbk::pdl_entry();
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ny) return;
  P3MCorners<D, G> cs;
  p3m_corners<D, G>(y + i * D, g, cs);
  if constexpr (std::is_same<G, float>::value) {
    if (dvp % 4 == 0 || dvp == 2) {
      for (int k0 = 0; k0 < dv; k0 += 4) {
        float wk[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) wk[q] = k0 + q < dv ? (float)wts[i * dv + k0 + q] : 0.f;
#pragma unroll
        for (int c = 0; c < (1 << D); ++c) {
          if (!(cs.use[c] && cs.interior[c])) continue;
          float *cell = grids + cs.l[c] * dvp + k0;
          const float wc = cs.w[c];
          if (dvp == 2)
            atomicAdd(reinterpret_cast<float2 *>(cell), make_float2(wc * wk[0], wc * wk[1]));
          else
            atomicAdd(reinterpret_cast<float4 *>(cell), make_float4(wc * wk[0], wc * wk[1], wc * wk[2], wc * wk[3]));
        }
      }
      return;
    }
  }
  for (int k = 0; k < dv; ++k) {
    const G wk = (G)wts[i * dv + k];
#pragma unroll
    for (int c = 0; c < (1 << D); ++c)
      if (cs.use[c] && cs.interior[c]) atomicAdd(grids + cs.l[c] * dvp + k, cs.w[c] * wk);
  }
}

// out[img] = spec[grid_of(img)] * kspec[kernel_of(img)] / N for img < nimg
template <typename C, typename G>
__global__ void p3m_multiply(const C *spec, const C *kspec, int nimg, int per_grid, int kernel0, long ccells, G scale,
                             C *out) {
  gbk::pdl_entry();
  long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ccells) return;
  for (int m = 0; m < nimg; ++m) {
    const C a = spec[(long)(m / per_grid) * ccells + j];
    const C b = kspec[(long)(kernel0 + m % per_grid) * ccells + j];
    C r;
    r.x = (a.x * b.x - a.y * b.y) * scale;
    r.y = (a.x * b.y + a.y * b.x) * scale;
    out[(long)m * ccells + j] = r;
  }
}

// Interleaved weight grids (cell-major, dvp slots per cell, as the splat's vector atomics write them)
// to the contiguous grids the forward transform reads (cuFFT's strided real layouts measured 2.4x
// slower for the forward and 8.5x for the inverse transform than its contiguous ones on 128^3
// grids, so the transforms and the interpolation's images stay contiguous).
template <typename G>
__global__ void p3m_deinterleave(const G *in, long cells, int dv, int dvp, G *out) {
  gbk::pdl_entry();
  const long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cells) return;
  for (int k = 0; k < dv; ++k) out[(long)k * cells + j] = in[j * dvp + k];
}

// values at the targets: mode 0 the nimg images; mode 2 contracted with alpha (images ordered
// p + D k, out nx x D); mode 3 the symmetric Hessians (images ordered q + D(D+1)/2 k, q the upper
// entry, out nx x dv x D x D). Sums in the grid's precision G.
template <int D, typename G>
__global__ void p3m_interp(const double *x, long nx, const G *imgs, int nimg, long cells, P3MGrid g, int mode,
                           const double *alpha, int dv, double *out) {
  gbk::pdl_entry();
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx) return;
  P3MCorners<D, G> cs;
  p3m_corners<D, G>(x + i * D, g, cs);
  if (mode == 0) {
    for (int q = 0; q < nimg; ++q) {
      G v = (G)0;
#pragma unroll
      for (int c = 0; c < (1 << D); ++c)
        if (cs.use[c]) v += cs.w[c] * imgs[(long)q * cells + cs.l[c]];
      out[i * nimg + q] = (double)v;
    }
  } else if (mode == 3) {
    constexpr int H = D * (D + 1) / 2;
    for (int k = 0; k < dv; ++k) {
      int q = 0;
      for (int r = 0; r < D; ++r)
        for (int cc = r; cc < D; ++cc, ++q) {
          G v = (G)0;
#pragma unroll
          for (int c = 0; c < (1 << D); ++c)
            if (cs.use[c]) v += cs.w[c] * imgs[(long)(q + H * k) * cells + cs.l[c]];
          out[((i * dv + k) * D + r) * D + cc] = (double)v;
          out[((i * dv + k) * D + cc) * D + r] = (double)v;
        }
    }
  } else {
    G r[D];
#pragma unroll
    for (int p = 0; p < D; ++p) r[p] = (G)0;
    for (int k = 0; k < dv; ++k) {
      const G a = (G)alpha[i * dv + k];
#pragma unroll
      for (int p = 0; p < D; ++p) {
        G v = (G)0;
#pragma unroll
        for (int c = 0; c < (1 << D); ++c)
          if (cs.use[c]) v += cs.w[c] * imgs[(long)(p + D * k) * cells + cs.l[c]];
        r[p] += v * a;
      }
    }
#pragma unroll
    for (int p = 0; p < D; ++p) out[i * D + p] = (double)r[p];
  }
}

// bounding box of x and y: one CTA, FP64
template <int D>
__global__ void p3m_box(const double *x, long nx, const double *y, long ny, double *box) {
  gbk::pdl_entry();
  __shared__ double s_lo[D][256], s_hi[D][256];
  double lo[D], hi[D];
  for (int k = 0; k < D; ++k) {
    lo[k] = 1e300;
    hi[k] = -1e300;
  }
  for (long i = threadIdx.x; i < nx + ny; i += blockDim.x) {
    const double *p = i < nx ? x + i * D : y + (i - nx) * D;
    for (int k = 0; k < D; ++k) {
      lo[k] = fmin(lo[k], p[k]);
      hi[k] = fmax(hi[k], p[k]);
    }
  }
  for (int k = 0; k < D; ++k) {
    s_lo[k][threadIdx.x] = lo[k];
    s_hi[k][threadIdx.x] = hi[k];
  }
  __syncthreads();
  for (int st = blockDim.x / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st)
      for (int k = 0; k < D; ++k) {
        s_lo[k][threadIdx.x] = fmin(s_lo[k][threadIdx.x], s_lo[k][threadIdx.x + st]);
        s_hi[k][threadIdx.x] = fmax(s_hi[k][threadIdx.x], s_hi[k][threadIdx.x + st]);
      }
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < D; ++k) {
      box[k] = s_lo[k][0];
      box[D + k] = s_hi[k][0];
    }
}

int fft_error(gbk_ctx *c, cufftResult r, const char *what) {
  return r == CUFFT_SUCCESS ? GBK_OK : c->fail(GBK_ERR_CUDA, "cuFFT %s failed (%d)", what, (int)r);
}

template <typename G>
struct P3MFFT;
template <>
struct P3MFFT<double> {
  typedef cufftDoubleComplex C;
  static constexpr cufftType R2C = CUFFT_D2Z, C2R = CUFFT_Z2D;
  static cufftResult fwd(cufftHandle h, double *in, C *out) { return cufftExecD2Z(h, in, out); }
  static cufftResult inv(cufftHandle h, C *in, double *out) { return cufftExecZ2D(h, in, out); }
};
template <>
struct P3MFFT<float> {
  typedef cufftComplex C;
  static constexpr cufftType R2C = CUFFT_R2C, C2R = CUFFT_C2R;
  static cufftResult fwd(cufftHandle h, float *in, C *out) { return cufftExecR2C(h, in, out); }
  static cufftResult inv(cufftHandle h, C *in, float *out) { return cufftExecC2R(h, in, out); }
};

// a cached batched plan over `batch` contiguous grids of g (real distance cells, complex ccells)
int p3m_plan(gbk_ctx *c, P3MCache *pc, const P3MGrid &g, cufftType type, int batch, cufftHandle *out) {
  for (const P3MPlan &p : pc->plans)
    if (p.type == type && p.batch == batch) {
      *out = p.h;
      return fft_error(c, cufftSetStream(p.h, c->stream), "stream");
    }
  int n[3] = {(int)g.n[0], (int)g.n[1], (int)g.n[2]};
  cufftHandle h;
  const cufftResult r = cufftPlanMany(&h, g.d, n, nullptr, 1, 0, nullptr, 1, 0, type, batch);
  if (r != CUFFT_SUCCESS) return fft_error(c, r, "plan");
  pc->plans.push_back({type, batch, h});
  *out = h;
  return fft_error(c, cufftSetStream(h, c->stream), "stream");
}

// Interleaved width of the splat's weight grids: cell-major with this many slots per cell (the weight
// count rounded up to 4 from 3 on, to 2 for 2), so that one vector atomic adds a source's weights into
// a cell (the scalar atomics of a planar layout were the splat's cost).
inline int p3m_slots(int n) { return n <= 1 ? 1 : n == 2 ? 2 : (n + 3) / 4 * 4; }

size_t up256(size_t b) { return (b + 255) & ~(size_t)255; }

// kernel spectra (cached), splat, one batched forward transform, spectrum products, one batched
// inverse transform, interpolation
template <typename G>
int p3m_exec(gbk_ctx *c, P3MCache *pc, const P3MGrid &g, int mode, int p0, int p1, int dv, const double *dx, long nx,
             const double *dy, const double *dw, long ny, double sigma, const double *da, double *dout, HostIO &io) {
  typedef typename P3MFFT<G>::C C;
  const int d = g.d, nk = p3m_kernels(d), H = d * (d + 1) / 2;
  cudaStream_t st = c->stream;
  const long cells = g.cells(), ccells = g.ccells();
  // images per weight grid and the first kernel they use, and the interpolation's output form
  int per_grid = 1, kernel0 = 0, interp = 0;
  switch (mode) {
    case 1: per_grid = d, kernel0 = 1; break;                  // ConvolveGradient(X)
    case 2: per_grid = d, kernel0 = 1, interp = 2; break;      // ConvolveGradient(X, alpha)
    case 3: kernel0 = 1 + p0; break;                           // ConvolveGradient(X, dim)
    case 4: per_grid = H, kernel0 = 1 + d, interp = 3; break;  // ConvolveHessian(X)
    case 5: {                                                  // ConvolveHessian(X, row, col)
      const int r = std::min(p0, p1), cc = std::max(p0, p1);
      kernel0 = 1 + d + cc + d * r - r * (r + 1) / 2;
      break;
    }
    default: break;                                            // Convolve
  }
  const int nimg = dv * per_grid;
  const bool f64 = sizeof(G) == 8;
  int rc = 0;
  if (!(pc->valid && pc->s == g.s && pc->sigma == sigma && pc->f64 == f64)) {
    pc->valid = false;
    if (pc->kspec) {
      cudaStreamSynchronize(st);
      cudaFree(pc->kspec);
      pc->kspec = nullptr;
    }
    cufftHandle kp;
    if ((rc = p3m_plan(c, pc, g, P3MFFT<G>::R2C, nk, &kp))) return rc;
    if ((rc = c->cuda(cudaMalloc(&pc->kspec, (size_t)ccells * nk * sizeof(C)), "cudaMalloc (P3M)"))) return rc;
    if ((rc = p3m_work(c, pc, (size_t)cells * nk * sizeof(G)))) return rc;
    G *kimg = (G *)pc->work;
    if (d == 3)
      p3m_kernel_images<3, G><<<nblk(cells), 256, 0, st>>>(g, sigma, kimg, cells);
    else
      p3m_kernel_images<2, G><<<nblk(cells), 256, 0, st>>>(g, sigma, kimg, cells);
    c->launches += 1;
    if ((rc = c->cuda(cudaGetLastError(), "kernel images"))) return rc;
    if ((rc = fft_error(c, P3MFFT<G>::fwd(kp, kimg, (C *)pc->kspec), "forward"))) return rc;
    pc->valid = true;
    pc->s = g.s;
    pc->sigma = sigma;
    pc->f64 = f64;
  }
  cufftHandle fwd, inv;
  const int dvp = p3m_slots(dv);
  if ((rc = p3m_plan(c, pc, g, P3MFFT<G>::R2C, dv, &fwd))) return rc;
  if ((rc = p3m_plan(c, pc, g, P3MFFT<G>::C2R, nimg, &inv))) return rc;
  const size_t b_spec = up256((size_t)ccells * dv * sizeof(C)), b_prod = up256((size_t)ccells * nimg * sizeof(C));
  const size_t b_grid = up256((size_t)cells * dv * sizeof(G)), b_img = up256((size_t)cells * nimg * sizeof(G));
  const size_t b_igrid = up256((size_t)cells * dvp * sizeof(G));
  if ((rc = p3m_work(c, pc, b_spec + b_prod + b_grid + b_img + b_igrid))) return rc;
  char *base = (char *)pc->work;
  C *spec = (C *)base;
  C *prod = (C *)(base + b_spec);
  G *grids = (G *)(base + b_spec + b_prod);
  G *imgs = (G *)(base + b_spec + b_prod + b_grid);
  G *igrids = (G *)(base + b_spec + b_prod + b_grid + b_img);  // the splat's interleaved grids
  rc = c->cuda(cudaMemsetAsync(igrids, 0, (size_t)cells * dvp * sizeof(G), st), "memset");
  if (!rc) {
    if (d == 3)
      p3m_splat<3, G><<<nblk(ny), 256, 0, st>>>(dy, dw, ny, dv, dvp, g, igrids);
    else
      p3m_splat<2, G><<<nblk(ny), 256, 0, st>>>(dy, dw, ny, dv, dvp, g, igrids);
    p3m_deinterleave<G><<<nblk(cells), 256, 0, st>>>(igrids, cells, dv, dvp, grids);
    c->launches += 2;
    rc = c->cuda(cudaGetLastError(), "splat");
  }
  if (!rc) rc = fft_error(c, P3MFFT<G>::fwd(fwd, grids, spec), "forward");
  if (!rc) {
    p3m_multiply<C, G><<<nblk(ccells), 256, 0, st>>>(spec, (const C *)pc->kspec, nimg, per_grid, kernel0, ccells,
                                                    (G)(1.0 / (double)cells), prod);
    c->launches += 1;
    rc = c->cuda(cudaGetLastError(), "multiply");
  }
  if (!rc) rc = fft_error(c, P3MFFT<G>::inv(inv, prod, imgs), "inverse");
  if (!rc) {
    if (d == 3)
      p3m_interp<3, G><<<nblk(nx), 256, 0, st>>>(dx, nx, imgs, nimg, cells, g, interp, da, dv, dout);
    else
      p3m_interp<2, G><<<nblk(nx), 256, 0, st>>>(dx, nx, imgs, nimg, cells, g, interp, da, dv, dout);
    c->launches += 1;
    rc = c->cuda(cudaGetLastError(), "interpolate");
  }
  if (!rc) rc = io.finish();
  if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
  cudaStreamSynchronize(st);  // the scratch is reused by the next call
  return rc;
}

// mode 0 Convolve (out nx x dv), 1 ConvolveGradient(X) (out nx x dv x d), 2 alpha-contracted (nx x d)
int p3m_run(gbk_ctx *c, int mode, int p0, int p1, int d, int dv, const double *x, long nx, const double *y,
            const double *w, long ny, double sigma, const double *alpha, const double *domain, double ratio,
            double padding, double *out) {
  if (!c) return GBK_ERR_ARG;
  c->err.clear();
  static const char *const kNames[6] = {"gbk_p3m_convolve",          "gbk_p3m_convolve_gradient",
                                        "gbk_p3m_convolve_gradient_alpha", "gbk_p3m_convolve_gradient_dim",
                                        "gbk_p3m_convolve_hessian",  "gbk_p3m_convolve_hessian_rowcol"};
  GbkRange range(kNames[mode < 0 || mode > 5 ? 0 : mode]);
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "P3M needs d = 2 or 3");
  if (nx <= 0 || ny <= 0 || dv <= 0) return c->fail(GBK_ERR_ARG, "empty input");
  if (!x || !y || !w || !out || (mode == 2 && !alpha)) return c->fail(GBK_ERR_ARG, "null pointer");
  if (!(sigma > 1e-20) || !(ratio > 0) || !(padding >= 0)) return c->fail(GBK_ERR_ARG, "bad P3M parameters");
  if (mode == 3 && (p0 < 0 || p0 >= d)) return c->fail(GBK_ERR_ARG, "dimension parameter out of bounds");
  if (mode == 5 && (p0 < 0 || p0 >= d || p1 < 0 || p1 >= d)) return c->fail(GBK_ERR_ARG, "dimension index out of bounds");
  if (c->capturing()) return c->fail(GBK_ERR_STATE, "P3M allocates and plans FFTs; not under stream capture");
  cudaStream_t st = c->stream;
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  const double *da = mode == 2 ? io.in(alpha, (size_t)nx * dv, "alpha") : nullptr;
  const size_t nout = (size_t)nx * (mode == 1 ? dv * d : mode == 2 ? d : mode == 4 ? dv * d * d : dv);
  double *dout = io.out(out, nout, "out");
  int rc = io.rc;
  if (rc) return rc;
  // the data domain: given, or the bounding box of targets and sources
  P3MCache *pc = (P3MCache *)c->p3m;
  if (!pc) {
    pc = new P3MCache();
    c->p3m = pc;
    c->p3m_free = p3m_cache_free;
  }
  double box[6];
  if (domain) {
    for (int k = 0; k < 2 * d; ++k) box[k] = domain[k];
  } else {
    rc = p3m_work(c, pc, 6 * sizeof(double));
    if (!rc) {
      double *dbox = (double *)pc->work;
      if (d == 3)
        p3m_box<3><<<1, 256, 0, st>>>(dx, nx, dy, ny, dbox);
      else
        p3m_box<2><<<1, 256, 0, st>>>(dx, nx, dy, ny, dbox);
      c->launches += 1;
      rc = c->cuda(cudaMemcpyAsync(box, dbox, 2 * d * sizeof(double), cudaMemcpyDeviceToHost, st), "read box");
      if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
    }
    if (rc) return rc;
  }
  // DetermineGrids
  P3MGrid g;
  g.d = d;
  g.s = ratio * sigma;
  g.inv_s = 1.0 / g.s;
  for (int k = 0; k < d; ++k) {
    const double length = box[d + k] - box[k];
    const double nd = (length + 2 * padding * sigma) / g.s;
    if (!(nd < 1073741824.0)) return c->fail(GBK_ERR_ARG, "P3M grid of more than 2^30 points along an axis");
    long n = (long)nd;
    if (n < 1) n = 1;
    double l2 = std::log((double)n) / std::log(2.0);
    const long t = (long)l2;
    l2 = (l2 - t) > 0 ? t + 1 : t;
    n = (long)std::pow(2.0, l2);
    g.n[k] = n;
    g.origin[k] = box[k] - (n * g.s - length) / 2;
  }
  const long cells = g.cells(), ccells = g.ccells();
  const int nimg = dv * (mode == 1 || mode == 2 ? d : mode == 4 ? d * (d + 1) / 2 : 1), nk = p3m_kernels(d);
  const bool f64 = c->mode == GBK_MODE_F64;
  const double re = f64 ? 8.0 : 4.0;  // grids, images, spectra, products, kernel spectra, cuFFT work areas
  const double bytes = re * cells * (dv + nimg) + 2 * re * ccells * (dv + nimg + nk + std::max(nimg, nk));
  if (bytes > 64e9) return c->fail(GBK_ERR_ARG, "P3M grid of %ld points needs %.0f GB", cells, bytes / 1e9);
  if (!(pc->d == d && pc->n[0] == g.n[0] && pc->n[1] == g.n[1] && pc->n[2] == g.n[2])) {
    cudaStreamSynchronize(st);
    pc->drop_plans();
    pc->valid = false;
    pc->d = d;
    for (int k = 0; k < 3; ++k) pc->n[k] = g.n[k];
  }
  return f64 ? p3m_exec<double>(c, pc, g, mode, p0, p1, dv, dx, nx, dy, dw, ny, sigma, da, dout, io)
             : p3m_exec<float>(c, pc, g, mode, p0, p1, dv, dx, nx, dy, dw, ny, sigma, da, dout, io);
}

}  // namespace

extern "C" {

int gbk_p3m_convolve(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y, const double *w, long ny,
                     double sigma, const double *domain, double spacing_ratio, double padding_factor, double *out) {
  return p3m_run(c, 0, 0, 0, d, dv, x, nx, y, w, ny, sigma, nullptr, domain, spacing_ratio, padding_factor, out);
}

int gbk_p3m_convolve_gradient(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y, const double *w,
                              long ny, double sigma, const double *domain, double spacing_ratio, double padding_factor,
                              double *out) {
  return p3m_run(c, 1, 0, 0, d, dv, x, nx, y, w, ny, sigma, nullptr, domain, spacing_ratio, padding_factor, out);
}

int gbk_p3m_convolve_gradient_alpha(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y,
                                    const double *w, long ny, double sigma, const double *alpha, const double *domain,
                                    double spacing_ratio, double padding_factor, double *out) {
  return p3m_run(c, 2, 0, 0, d, dv, x, nx, y, w, ny, sigma, alpha, domain, spacing_ratio, padding_factor, out);
}

int gbk_p3m_convolve_gradient_dim(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y,
                                  const double *w, long ny, double sigma, int dim, const double *domain,
                                  double spacing_ratio, double padding_factor, double *out) {
  return p3m_run(c, 3, dim, 0, d, dv, x, nx, y, w, ny, sigma, nullptr, domain, spacing_ratio, padding_factor, out);
}

int gbk_p3m_convolve_hessian(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y, const double *w,
                             long ny, double sigma, const double *domain, double spacing_ratio, double padding_factor,
                             double *out) {
  return p3m_run(c, 4, 0, 0, d, dv, x, nx, y, w, ny, sigma, nullptr, domain, spacing_ratio, padding_factor, out);
}

int gbk_p3m_convolve_hessian_rowcol(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y,
                                    const double *w, long ny, double sigma, int row, int col, const double *domain,
                                    double spacing_ratio, double padding_factor, double *out) {
  return p3m_run(c, 5, row, col, d, dv, x, nx, y, w, ny, sigma, nullptr, domain, spacing_ratio, padding_factor,
                 out);
}

// P3MKernel::ConvolveGradient(X, k, dp) and ConvolveHessian(X, k, dp, dq) (P3MKernel.cxx:1506-1547,
// 1689-1729) check their indices and return nx zeros.
static int p3m_zeros(gbk_ctx *c, int d, int dv, long nx, long ny, int k, int dp, int dq, double *out) {
  if (!c) return GBK_ERR_ARG;
  c->err.clear();
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "P3M needs d = 2 or 3");
  if (nx < 0 || ny < 0 || dv <= 0) return c->fail(GBK_ERR_ARG, "bad sizes");
  if (k < 0 || k >= dv) return c->fail(GBK_ERR_ARG, "Invalid weight index");
  if (dp < 0 || dp >= d || dq < 0 || dq >= d) return c->fail(GBK_ERR_ARG, "Invalid derivative direction");
  if (nx == 0) return GBK_OK;
  if (!out) return c->fail(GBK_ERR_ARG, "null pointer");
  bool dev = false;
  if (int rc = locate(c, out, "out", &dev)) return rc;
  if (dev) {
    if (int rc = c->cuda(cudaMemsetAsync(out, 0, (size_t)nx * sizeof(double), c->stream), "memset")) return rc;
    return c->cuda(cudaStreamSynchronize(c->stream), "sync");
  }
  std::fill(out, out + nx, 0.0);
  return GBK_OK;
}

int gbk_p3m_convolve_gradient_kdp(gbk_ctx *c, int d, int dv, long nx, long ny, int k, int dp, double *out) {
  return p3m_zeros(c, d, dv, nx, ny, k, dp, 0, out);
}

int gbk_p3m_convolve_hessian_kdpdq(gbk_ctx *c, int d, int dv, long nx, long ny, int k, int dp, int dq, double *out) {
  return p3m_zeros(c, d, dv, nx, ny, k, dp, dq, out);
}

}  // extern "C"
