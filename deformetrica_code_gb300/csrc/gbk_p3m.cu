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
// Everything is FP64. The splat accumulates with atomic adds (grid sums in arbitrary order, last-bit
// differences between runs); plans and kernel spectra are cached in the context per grid and width.
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
  long cells() const { return n[0] * n[1] * (d == 3 ? n[2] : 1); }
  long ccells() const { return n[0] * (d == 3 ? n[1] * (n[2] / 2 + 1) : (n[1] / 2 + 1)); }
};

struct P3MCache {
  bool valid = false;
  int d = 0;
  long n[3] = {0, 0, 0};
  double s = 0, sigma = 0;
  cufftHandle fwd = 0, inv = 0;
  bool plans = false;
  cufftDoubleComplex *kspec = nullptr;  // (1 + d) kernel spectra: Gaussian, then its gradient components
};

void p3m_cache_free(void *p) {
  P3MCache *c = (P3MCache *)p;
  if (!c) return;
  if (c->plans) {
    cufftDestroy(c->fwd);
    cufftDestroy(c->inv);
  }
  if (c->kspec) cudaFree(c->kspec);
  delete c;
}

unsigned nblk(long n, int bs = 256) { return (unsigned)std::max(1L, (n + bs - 1) / bs); }

template <int D>
__device__ inline long lin(const long *ind, const long *n) {
  return D == 3 ? (ind[0] * n[1] + ind[1]) * n[2] + ind[2] : ind[0] * n[1] + ind[1];
}

// Kernel images in inverse-FFT-shifted layout: slot j holds the value at grid index (j + n/2) mod n.
template <int D>
__global__ void p3m_kernel_images(P3MGrid g, double sigma, double *img, long cells) {
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
  const double kv = exp(-d2 / (sigma * sigma));
  img[j] = border ? 0.0 : kv;
  for (int k = 0; k < D; ++k) img[(1 + k) * cells + j] = border ? 0.0 : diff[k] * (-2.0 * kv / (sigma * sigma));
}

// multilinear corners of one point: returns their count, in the reference's order (first
// dimension slowest), outside points and zero weights dropped
template <int D>
__device__ inline int p3m_corners(const double *p, const P3MGrid &g, long (*ind)[3], double *w) {
  long i1[3];
  double f[3], h[3];
  for (int k = 0; k < D; ++k) {
    const double c = (p[k] - g.origin[k]) / g.s;
    i1[k] = (long)floor(c);
    f[k] = c - i1[k];
    h[k] = (i1[k] + 1) - c;
  }
  int m = 0;
  for (int b = 0; b < (1 << D); ++b) {
    double wt = 1.0;
    bool in = true;
    for (int k = 0; k < D; ++k) {
      const int bit = (b >> (D - 1 - k)) & 1;
      const long q = i1[k] + bit;
      wt *= bit ? f[k] : h[k];
      in = in && q >= 0 && q < g.n[k];
      ind[m][k] = q;
    }
    if (in && wt > 0) w[m++] = wt;
  }
  return m;
}

template <int D>
__global__ void p3m_splat(const double *y, const double *wts, long ny, int dv, P3MGrid g, double *grids, long cells) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ny) return;
  long ind[1 << D][3];
  double w[1 << D];
  const int m = p3m_corners<D>(y + i * D, g, ind, w);
  for (int c = 0; c < m; ++c) {
    bool border = false;
    for (int k = 0; k < D; ++k) border = border || ind[c][k] <= 0;
    if (border) continue;
    const long l = lin<D>(ind[c], g.n);
    for (int k = 0; k < dv; ++k) atomicAdd(grids + (long)k * cells + l, w[c] * wts[i * dv + k]);
  }
}

// out[img] = spec[grid_of(img)] * kspec[kernel_of(img)] / N for img < nimg
__global__ void p3m_multiply(const cufftDoubleComplex *spec, const cufftDoubleComplex *kspec, int nimg, int per_grid,
                             int kernel0, long ccells, double scale, cufftDoubleComplex *out) {
  long j = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ccells) return;
  for (int m = 0; m < nimg; ++m) {
    const cufftDoubleComplex a = spec[(long)(m / per_grid) * ccells + j];
    const cufftDoubleComplex b = kspec[(long)(kernel0 + m % per_grid) * ccells + j];
    out[(long)m * ccells + j] = make_cuDoubleComplex((a.x * b.x - a.y * b.y) * scale, (a.x * b.y + a.y * b.x) * scale);
  }
}

// values at the targets: mode 0 the nimg images; mode 2 contracted with alpha (images ordered
// p + D k, out nx x D)
template <int D>
__global__ void p3m_interp(const double *x, long nx, const double *imgs, int nimg, long cells, P3MGrid g, int mode,
                           const double *alpha, int dv, double *out) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx) return;
  long ind[1 << D][3];
  double w[1 << D];
  const int m = p3m_corners<D>(x + i * D, g, ind, w);
  long l[1 << D];
  for (int c = 0; c < m; ++c) l[c] = lin<D>(ind[c], g.n);
  if (mode == 0) {
    for (int q = 0; q < nimg; ++q) {
      double v = 0.0;
      for (int c = 0; c < m; ++c) v += w[c] * imgs[(long)q * cells + l[c]];
      out[i * nimg + q] = v;
    }
  } else {
    double r[3] = {0, 0, 0};
    for (int k = 0; k < dv; ++k)
      for (int p = 0; p < D; ++p) {
        double v = 0.0;
        for (int c = 0; c < m; ++c) v += w[c] * imgs[(long)(p + D * k) * cells + l[c]];
        r[p] += v * alpha[i * dv + k];
      }
    for (int p = 0; p < D; ++p) out[i * D + p] = r[p];
  }
}

// bounding box of x and y: one CTA, FP64
template <int D>
__global__ void p3m_box(const double *x, long nx, const double *y, long ny, double *box) {
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

// mode 0 Convolve (out nx x dv), 1 ConvolveGradient(X) (out nx x dv x d), 2 alpha-contracted (nx x d)
int p3m_run(gbk_ctx *c, int mode, int d, int dv, const double *x, long nx, const double *y, const double *w, long ny,
            double sigma, const double *alpha, const double *domain, double ratio, double padding, double *out) {
  if (!c) return GBK_ERR_ARG;
  c->err.clear();
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "P3M needs d = 2 or 3");
  if (nx <= 0 || ny <= 0 || dv <= 0) return c->fail(GBK_ERR_ARG, "empty input");
  if (!x || !y || !w || !out || (mode == 2 && !alpha)) return c->fail(GBK_ERR_ARG, "null pointer");
  if (!(sigma > 1e-20) || !(ratio > 0) || !(padding >= 0)) return c->fail(GBK_ERR_ARG, "bad P3M parameters");
  if (c->capturing()) return c->fail(GBK_ERR_STATE, "P3M allocates and plans FFTs; not under stream capture");
  cudaStream_t st = c->stream;
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  const double *da = mode == 2 ? io.in(alpha, (size_t)nx * dv, "alpha") : nullptr;
  const size_t nout = (size_t)nx * (mode == 0 ? dv : mode == 1 ? dv * d : d);
  double *dout = io.out(out, nout, "out");
  int rc = io.rc;
  if (rc) return rc;
  // the data domain: given, or the bounding box of targets and sources
  double box[6];
  if (domain) {
    for (int k = 0; k < 2 * d; ++k) box[k] = domain[k];
  } else {
    double *dbox = nullptr;
    rc = c->cuda(cudaMalloc(&dbox, 6 * sizeof(double)), "cudaMalloc");
    if (!rc) {
      if (d == 3)
        p3m_box<3><<<1, 256, 0, st>>>(dx, nx, dy, ny, dbox);
      else
        p3m_box<2><<<1, 256, 0, st>>>(dx, nx, dy, ny, dbox);
      c->launches += 1;
      rc = c->cuda(cudaMemcpyAsync(box, dbox, 2 * d * sizeof(double), cudaMemcpyDeviceToHost, st), "read box");
      if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
    }
    if (dbox) cudaFree(dbox);
    if (rc) return rc;
  }
  // DetermineGrids
  P3MGrid g;
  g.d = d;
  g.s = ratio * sigma;
  for (int k = 0; k < d; ++k) {
    const double length = box[d + k] - box[k];
    long n = (long)((length + 2 * padding * sigma) / g.s);
    if (n < 1) n = 1;
    double l2 = std::log((double)n) / std::log(2.0);
    const long t = (long)l2;
    l2 = (l2 - t) > 0 ? t + 1 : t;
    n = (long)std::pow(2.0, l2);
    g.n[k] = n;
    g.origin[k] = box[k] - (n * g.s - length) / 2;
  }
  const long cells = g.cells(), ccells = g.ccells();
  const int nimg = mode == 0 ? dv : dv * d;
  const double bytes = 8.0 * cells * (dv + nimg) + 16.0 * ccells * (dv + nimg + 1 + d);
  if (bytes > 64e9) return c->fail(GBK_ERR_ARG, "P3M grid of %ld points needs %.0f GB", cells, bytes / 1e9);
  // plans and kernel spectra, cached per grid size, spacing and width
  P3MCache *pc = (P3MCache *)c->p3m;
  if (!pc) {
    pc = new P3MCache();
    c->p3m = pc;
    c->p3m_free = p3m_cache_free;
  }
  const bool same = pc->valid && pc->d == d && pc->n[0] == g.n[0] && pc->n[1] == g.n[1] &&
                    (d == 2 || pc->n[2] == g.n[2]) && pc->s == g.s && pc->sigma == sigma;
  if (!same) {
    if (pc->plans) {
      cufftDestroy(pc->fwd);
      cufftDestroy(pc->inv);
      pc->plans = false;
    }
    if (pc->kspec) cudaFree(pc->kspec);
    pc->kspec = nullptr;
    pc->valid = false;
    cufftResult fr = d == 3 ? cufftPlan3d(&pc->fwd, (int)g.n[0], (int)g.n[1], (int)g.n[2], CUFFT_D2Z)
                            : cufftPlan2d(&pc->fwd, (int)g.n[0], (int)g.n[1], CUFFT_D2Z);
    if ((rc = fft_error(c, fr, "plan"))) return rc;
    fr = d == 3 ? cufftPlan3d(&pc->inv, (int)g.n[0], (int)g.n[1], (int)g.n[2], CUFFT_Z2D)
                : cufftPlan2d(&pc->inv, (int)g.n[0], (int)g.n[1], CUFFT_Z2D);
    if ((rc = fft_error(c, fr, "plan"))) {
      cufftDestroy(pc->fwd);
      return rc;
    }
    pc->plans = true;
    double *kimg = nullptr;
    rc = c->cuda(cudaMalloc(&kimg, (size_t)cells * (1 + d) * sizeof(double)), "cudaMalloc (P3M)");
    if (!rc) rc = c->cuda(cudaMalloc(&pc->kspec, (size_t)ccells * (1 + d) * sizeof(cufftDoubleComplex)), "cudaMalloc (P3M)");
    if (!rc) {
      if (d == 3)
        p3m_kernel_images<3><<<nblk(cells), 256, 0, st>>>(g, sigma, kimg, cells);
      else
        p3m_kernel_images<2><<<nblk(cells), 256, 0, st>>>(g, sigma, kimg, cells);
      c->launches += 1;
      rc = c->cuda(cudaGetLastError(), "kernel images");
    }
    for (int k = 0; k <= d && !rc; ++k) {
      rc = fft_error(c, cufftSetStream(pc->fwd, st), "stream");
      if (!rc) rc = fft_error(c, cufftExecD2Z(pc->fwd, kimg + (long)k * cells, pc->kspec + (long)k * ccells), "D2Z");
    }
    if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
    if (kimg) cudaFree(kimg);
    if (rc) return rc;
    pc->valid = true;
    pc->d = d;
    for (int k = 0; k < 3; ++k) pc->n[k] = g.n[k];
    pc->s = g.s;
    pc->sigma = sigma;
  }
  // splat, transform, multiply, transform back, interpolate
  double *grids = nullptr, *imgs = nullptr;
  cufftDoubleComplex *spec = nullptr, *prod = nullptr;
  rc = c->cuda(cudaMalloc(&grids, (size_t)cells * dv * sizeof(double)), "cudaMalloc (P3M)");
  if (!rc) rc = c->cuda(cudaMalloc(&imgs, (size_t)cells * nimg * sizeof(double)), "cudaMalloc (P3M)");
  if (!rc) rc = c->cuda(cudaMalloc(&spec, (size_t)ccells * dv * sizeof(cufftDoubleComplex)), "cudaMalloc (P3M)");
  if (!rc) rc = c->cuda(cudaMalloc(&prod, (size_t)ccells * nimg * sizeof(cufftDoubleComplex)), "cudaMalloc (P3M)");
  if (!rc) rc = c->cuda(cudaMemsetAsync(grids, 0, (size_t)cells * dv * sizeof(double), st), "memset");
  if (!rc) {
    if (d == 3)
      p3m_splat<3><<<nblk(ny), 256, 0, st>>>(dy, dw, ny, dv, g, grids, cells);
    else
      p3m_splat<2><<<nblk(ny), 256, 0, st>>>(dy, dw, ny, dv, g, grids, cells);
    c->launches += 1;
    rc = c->cuda(cudaGetLastError(), "splat");
  }
  if (!rc) rc = fft_error(c, cufftSetStream(pc->fwd, st), "stream");
  if (!rc) rc = fft_error(c, cufftSetStream(pc->inv, st), "stream");
  for (int k = 0; k < dv && !rc; ++k)
    rc = fft_error(c, cufftExecD2Z(pc->fwd, grids + (long)k * cells, spec + (long)k * ccells), "D2Z");
  if (!rc) {
    p3m_multiply<<<nblk(ccells), 256, 0, st>>>(spec, pc->kspec, nimg, mode == 0 ? 1 : d, mode == 0 ? 0 : 1, ccells,
                                               1.0 / (double)cells, prod);
    c->launches += 1;
    rc = c->cuda(cudaGetLastError(), "multiply");
  }
  for (int m = 0; m < nimg && !rc; ++m)
    rc = fft_error(c, cufftExecZ2D(pc->inv, prod + (long)m * ccells, imgs + (long)m * cells), "Z2D");
  if (!rc) {
    if (d == 3)
      p3m_interp<3><<<nblk(nx), 256, 0, st>>>(dx, nx, imgs, nimg, cells, g, mode == 2 ? 2 : 0, da, dv, dout);
    else
      p3m_interp<2><<<nblk(nx), 256, 0, st>>>(dx, nx, imgs, nimg, cells, g, mode == 2 ? 2 : 0, da, dv, dout);
    c->launches += 1;
    rc = c->cuda(cudaGetLastError(), "interpolate");
  }
  if (!rc) rc = io.finish();
  if (!rc) rc = c->cuda(cudaStreamSynchronize(st), "sync");
  cudaStreamSynchronize(st);
  for (void *p : {(void *)grids, (void *)imgs, (void *)spec, (void *)prod})
    if (p) cudaFree(p);
  return rc;
}

}  // namespace

extern "C" {

int gbk_p3m_convolve(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y, const double *w, long ny,
                     double sigma, const double *domain, double spacing_ratio, double padding_factor, double *out) {
  return p3m_run(c, 0, d, dv, x, nx, y, w, ny, sigma, nullptr, domain, spacing_ratio, padding_factor, out);
}

int gbk_p3m_convolve_gradient(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y, const double *w,
                              long ny, double sigma, const double *domain, double spacing_ratio, double padding_factor,
                              double *out) {
  return p3m_run(c, 1, d, dv, x, nx, y, w, ny, sigma, nullptr, domain, spacing_ratio, padding_factor, out);
}

int gbk_p3m_convolve_gradient_alpha(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y,
                                    const double *w, long ny, double sigma, const double *alpha, const double *domain,
                                    double spacing_ratio, double padding_factor, double *out) {
  return p3m_run(c, 2, d, dv, x, nx, y, w, ny, sigma, alpha, domain, spacing_ratio, padding_factor, out);
}

}  // extern "C"
