// FP64 reductions (RKHS norm) and the autotuner of the kernel-sum launch parameters.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_dispatch.h"
#include "gbk_hostio.h"

using namespace gbk;

namespace gbk {

// sum_i a_i * b_i over n doubles in FP64, one CTA, fixed order: bitwise reproducible.
__global__ void __launch_bounds__(1024) dot_f64_kernel(const double *a, const double *b, long n,
                                                       double *out, int accumulate) {
  __shared__ double s[1024];
  double acc = 0.0;
  for (long i = threadIdx.x; i < n; i += blockDim.x) acc = fma(a[i], b[i], acc);
  s[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    if (accumulate)
      *out += s[0];
    else
      *out = s[0];
  }
}

// Synthetic inputs for tuning: uniform [0,1) coordinates / uniform [-1,1) weights (hash based).
__global__ void fill_uniform_kernel(double *p, long n, unsigned seed, double lo, double hi) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned long long z = (unsigned long long)i * 0x9E3779B97F4A7C15ull + seed * 0xD1B54A32D192ED03ull;
  z ^= z >> 31;
  z *= 0xBF58476D1CE4E5B9ull;
  z ^= z >> 29;
  z *= 0x94D049BB133111EBull;
  z ^= z >> 32;
  double u = (double)(z >> 11) * (1.0 / 9007199254740992.0);
  p[i] = lo + (hi - lo) * u;
}

}  // namespace gbk

extern "C" {

int gbk_kernel_norm(gbk_ctx *c, int d, int dv, const double *y, const double *w, long n,
                    double sigma, double *out) {
  if (!c) return GBK_ERR_ARG;
  c->err.clear();
  if (!out) return c->fail(GBK_ERR_ARG, "null output");
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  // K w into the context's temporary buffer, then <w, K w> in FP64
  int rc = c->ensure(c->tmp, (size_t)std::max(n, 1L) * dv * sizeof(double), "kernel norm temporary");
  if (rc) return rc;
  rc = c->ensure(c->reduce, 4 * sizeof(double), "kernel norm scalar");
  if (rc) return rc;
  // Inputs may be host pointers: gbk_convolve stages them; the reduction then needs w on the
  // device, so stage explicitly here.
  bool dev_w = false, dev_y = false, dev_out = false;
  if ((rc = locate(c, w, "w", &dev_w)) || (rc = locate(c, y, "y", &dev_y)) || (rc = locate(c, out, "out", &dev_out)))
    return rc;
  const double *dw = w, *dy = y;
  gbk_ctx::DevBuf &sw = c->stage[gbk_ctx::kStageSlots - 1];
  gbk_ctx::DevBuf &sy = c->stage[gbk_ctx::kStageSlots - 2];
  if (!dev_w && n) {
    if ((rc = c->ensure(sw, (size_t)n * dv * sizeof(double), "w"))) return rc;
    if ((rc = c->cuda(cudaMemcpyAsync(sw.p, w, (size_t)n * dv * sizeof(double), cudaMemcpyHostToDevice, c->stream), "H2D")))
      return rc;
    dw = (const double *)sw.p;
  }
  if (!dev_y && n) {
    if ((rc = c->ensure(sy, (size_t)n * d * sizeof(double), "y"))) return rc;
    if ((rc = c->cuda(cudaMemcpyAsync(sy.p, y, (size_t)n * d * sizeof(double), cudaMemcpyHostToDevice, c->stream), "H2D")))
      return rc;
    dy = (const double *)sy.p;
  }
  rc = gbk_convolve(c, d, dv, dy, n, dy, dw, n, sigma, (double *)c->tmp.p);
  if (rc) return rc;
  double *dst = dev_out ? out : (double *)c->reduce.p;
  dot_f64_kernel<<<1, 1024, 0, c->stream>>>(dw, (const double *)c->tmp.p, n * (long)dv, dst, 0);
  if ((rc = c->cuda(cudaGetLastError(), "dot_f64_kernel"))) return rc;
  c->launches += 1;
  if (!dev_out) {
    if ((rc = c->cuda(cudaMemcpyAsync(out, dst, sizeof(double), cudaMemcpyDeviceToHost, c->stream), "D2H"))) return rc;
    return c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
  }
  return GBK_OK;
}

int gbk_autotune(gbk_ctx *c, int op, int d, int dv, long nx, long ny, double sigma) {
  if (!c) return GBK_ERR_ARG;
  c->err.clear();
  if (op < 0 || op >= OP_COUNT) return c->fail(GBK_ERR_ARG, "unknown op %d", op);
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "dimension %d", d);
  if (nx <= 0 || ny <= 0) return c->fail(GBK_ERR_ARG, "autotune needs nx, ny > 0");
  if (op == OP_SPECIAL) {
    dv = d;
    ny = nx;
  }
  KernelEntry e0;
  if (!find_kernel(op, c->mode, d, dv, 0, &e0)) return c->fail(GBK_ERR_UNSUPPORTED, "op %d d=%d dv=%d", op, d, dv);
  if (c->capturing()) return c->fail(GBK_ERR_STATE, "autotune during stream capture");
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");

  const long nin = std::max(nx, ny);
  size_t sz_x = (size_t)nin * d, sz_w = (size_t)nin * 6, sz_o = (size_t)nx * dv * d * d + (size_t)nx * 16;
  std::vector<double *> bufs;
  auto alloc = [&](size_t n) -> double * {
    double *p = nullptr;
    if (cudaMalloc(&p, n * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    bufs.push_back(p);
    return p;
  };
  auto cleanup = [&]() {
    cudaStreamSynchronize(c->stream);
    for (double *p : bufs) cudaFree(p);
    cudaGetLastError();
  };
  double *X = alloc(sz_x), *Y = alloc(sz_x), *Wt = alloc(sz_w), *A = alloc(sz_w), *O0 = alloc(sz_o), *O1 = alloc((size_t)nx * d);
  if (!X || !Y || !Wt || !A || !O0 || !O1) {
    cleanup();
    return c->fail(GBK_ERR_ALLOC, "autotune buffers");
  }
  fill_uniform_kernel<<<(unsigned)((sz_x + 255) / 256), 256, 0, c->stream>>>(X, (long)sz_x, 1, 0.0, 1.0);
  fill_uniform_kernel<<<(unsigned)((sz_x + 255) / 256), 256, 0, c->stream>>>(Y, (long)sz_x, 2, 0.0, 1.0);
  fill_uniform_kernel<<<(unsigned)((sz_w + 255) / 256), 256, 0, c->stream>>>(Wt, (long)sz_w, 3, -1.0, 1.0);
  fill_uniform_kernel<<<(unsigned)((sz_w + 255) / 256), 256, 0, c->stream>>>(A, (long)sz_w, 4, -1.0, 1.0);

  PairArgs a;
  memset(&a, 0, sizeof a);
  a.x = X;
  a.nx = nx;
  a.y = (op == OP_SPECIAL) ? X : Y;
  a.ny = ny;
  a.w = Wt;
  a.w_ld = dv;
  a.ta = (op == OP_SPECIAL) ? Wt : A;
  a.ta_ld = dv;
  a.tb = A;
  a.tb_ld = d;
  a.sb = A;
  a.sb_ld = d;
  a.sigma = sigma < 1e-10 ? 1e-10 : sigma;
  a.out0 = O0;
  a.out0_ld = op_outputs(op, d, dv) + 8;
  a.out1 = O1;
  a.out1_ld = d;
  a.nsplit = 1;

  cudaEvent_t e_start, e_stop;
  cudaEventCreate(&e_start);
  cudaEventCreate(&e_stop);
  const auto k = c->key(op, d, dv, nx, ny);
  const int saved_force = c->force_split;
  c->force_split = 0;
  float best_ms = 1e30f;
  std::pair<int, int> best{0, 1};
  int rc = GBK_OK;
  const int nv = num_variants(op, c->mode, d, dv);
  for (int v = 0; v < nv && !rc; ++v) {
    KernelEntry e;
    if (!find_kernel(op, c->mode, d, dv, v, &e)) continue;
    std::vector<int> cands = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32};
    c->tune.erase(k);
    int heur = c->choose_split(e, d, nx, ny);
    cands.push_back(heur);
    std::sort(cands.begin(), cands.end());
    cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
    long max_split = std::max(1L, ny / (2L * e.tj));
    for (int ns : cands) {
      if (ns > max_split) continue;
      c->tune[k] = {v, ns};
      rc = c->launch(op, d, dv, a);  // warm-up
      if (rc) break;
      cudaEventRecord(e_start, c->stream);
      const int reps = 3;
      for (int r = 0; r < reps && !rc; ++r) rc = c->launch(op, d, dv, a);
      cudaEventRecord(e_stop, c->stream);
      if (rc) break;
      cudaEventSynchronize(e_stop);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e_start, e_stop);
      ms /= reps;
      if (ms < best_ms) {
        best_ms = ms;
        best = {v, ns};
      }
    }
  }
  c->force_split = saved_force;
  cudaEventDestroy(e_start);
  cudaEventDestroy(e_stop);
  cleanup();
  if (rc) {
    c->tune.erase(k);
    return rc;
  }
  c->tune[k] = best;
  return GBK_OK;
}

int gbk_tune_save(const gbk_ctx *c, const char *path) {
  if (!c || !path) return GBK_ERR_ARG;
  FILE *f = fopen(path, "w");
  if (!f) return GBK_ERR_ARG;
  for (const auto &kv : c->tune) {
    int op, mode, d, dv, bx, by;
    std::tie(op, mode, d, dv, bx, by) = kv.first;
    fprintf(f, "{\"op\": %d, \"mode\": %d, \"d\": %d, \"dv\": %d, \"bx\": %d, \"by\": %d, \"variant\": %d, \"nsplit\": %d}\n",
            op, mode, d, dv, bx, by, kv.second.first, kv.second.second);
  }
  fclose(f);
  return GBK_OK;
}

int gbk_tune_load(gbk_ctx *c, const char *path) {
  if (!c || !path) return GBK_ERR_ARG;
  FILE *f = fopen(path, "r");
  if (!f) return c->fail(GBK_ERR_ARG, "cannot open %s", path);
  char line[512];
  while (fgets(line, sizeof line, f)) {
    int op, mode, d, dv, bx, by, v, ns;
    if (sscanf(line, "{\"op\": %d, \"mode\": %d, \"d\": %d, \"dv\": %d, \"bx\": %d, \"by\": %d, \"variant\": %d, \"nsplit\": %d}",
               &op, &mode, &d, &dv, &bx, &by, &v, &ns) == 8) {
      if (v < 0 || (v >= num_variants(op, mode, d, dv) && v != VARIANT_SMALL) || ns < 0) continue;  // nsplit 0 = automatic
      c->tune[gbk_ctx::TuneKey{op, mode, d, dv, bx, by}] = {v, ns};
    }
  }
  fclose(f);
  return GBK_OK;
}

}  // extern "C"
