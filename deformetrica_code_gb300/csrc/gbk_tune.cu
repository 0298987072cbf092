// FP64 reductions (RKHS norm) and the autotuner of the kernel-sum launch parameters.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <tuple>
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
  if (threadIdx.x == 0) {
    if (accumulate)
      *out += s[0];
    else
      *out = s[0];
  }
}

// Synthetic inputs for tuning: uniform [0,1) coordinates / uniform [-1,1) weights (hash based).
__global__ void fill_uniform_kernel(double *p, long n, unsigned seed, double lo, double hi) {
  pdl_entry();
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

}  // extern "C"

namespace {

// Times every compiled variant of the launch's path (gbk_ctx::family) with a range of source-split
// counts through gbk_ctx::launch itself (the same order policy, sorts, staging and split reduction
// as the call being tuned) and keeps the fastest (variant, split) for the call's size bucket and
// path. `a` holds valid device arrays. The spatial order's sorts are made once (order cache).
int tune_core(gbk_ctx *c, int op, int d, int dv, PairArgs a, int *best_variant, int *best_split, float *best_ms_out) {
  gbk_ctx::OrderCacheScope cache(c);
  gbk_ctx::LaunchPlan pl;
  if (int rc = c->plan(op, d, dv, a, &pl)) return rc;
  const auto k = c->key(op, d, dv, a.nx, a.ny, pl.path);
  const std::vector<int> fam = c->family(pl.path, op, d, dv);
  if (fam.empty()) return c->fail(GBK_ERR_UNSUPPORTED, "op %d d=%d dv=%d", op, d, dv);
  cudaEvent_t e_start, e_stop;
  if (cudaEventCreate(&e_start) != cudaSuccess || cudaEventCreate(&e_stop) != cudaSuccess) {
    cudaGetLastError();
    return c->fail(GBK_ERR_CUDA, "cudaEventCreate");
  }
  const int saved_force = c->force_split;
  c->force_split = 0;
  const auto saved = c->tune.find(k) != c->tune.end() ? c->tune[k] : std::pair<int, int>{-1, -1};
  float best_ms = 1e30f;
  std::pair<int, int> best{pl.variant, 0};
  int rc = GBK_OK;
  for (int v : fam) {
    KernelEntry e;
    if (!find_kernel(op, c->mode, d, dv, v, &e)) continue;
    const long max_split = std::max(1L, a.ny / ((e.ks > 0 ? (long)e.ks : 2L) * e.tj));
    std::vector<int> cands = {1, 2, 3, 4, 6, 8, 12, 16, 24, 32};
    cands.push_back(c->choose_split(e, d, a.nx, a.ny));
    std::sort(cands.begin(), cands.end());
    cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
    bool warm = false;
    for (int ns : cands) {
      if (ns > max_split && ns != 1) continue;
      c->tune[k] = {v, ns};
      if (!warm) {  // first launch of the variant: module load, buffer growth, sorts
        if ((rc = c->launch(op, d, dv, a))) break;
        warm = true;
      }
      cudaEventRecord(e_start, c->stream);
      if ((rc = c->launch(op, d, dv, a))) break;
      cudaEventRecord(e_stop, c->stream);
      cudaEventSynchronize(e_stop);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e_start, e_stop);
      if (ms < 20.f) {  // short launches: the best of three
        for (int r = 0; r < 2 && !rc; ++r) {
          cudaEventRecord(e_start, c->stream);
          rc = c->launch(op, d, dv, a);
          cudaEventRecord(e_stop, c->stream);
          cudaEventSynchronize(e_stop);
          float m2 = 0.f;
          cudaEventElapsedTime(&m2, e_start, e_stop);
          ms = std::min(ms, m2);
        }
        if (rc) break;
      }
      if (ms < best_ms) {
        best_ms = ms;
        best = {v, ns};
      }
    }
    if (rc) break;
  }
  c->force_split = saved_force;
  cudaEventDestroy(e_start);
  cudaEventDestroy(e_stop);
  if (rc) {
    if (saved.first >= 0)
      c->tune[k] = saved;
    else
      c->tune.erase(k);
    return rc;
  }
  c->tune[k] = best;
  if (best_variant) *best_variant = best.first;
  if (best_split) *best_split = best.second;
  if (best_ms_out) *best_ms_out = best_ms;
  return GBK_OK;
}

bool tunable_op(int op) { return op >= OP_CONV && op <= OP_HESSRC; }

// device scratch of one tuning call (freed on every exit)
struct TuneBuffers {
  std::vector<double *> bufs;
  double *get(size_t n) {
    double *p = nullptr;
    if (cudaMalloc(&p, std::max(n, (size_t)1) * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    bufs.push_back(p);
    return p;
  }
  ~TuneBuffers() {
    cudaDeviceSynchronize();
    for (double *p : bufs) cudaFree(p);
    cudaGetLastError();
  }
};

PairArgs tune_args(int op, int d, int dv, const double *x, long nx, const double *y, const double *w, long ny,
                   double sigma, const double *alpha, double *o0, double *o1) {
  PairArgs a;
  memset(&a, 0, sizeof a);
  a.x = x;
  a.nx = nx;
  a.y = y;
  a.ny = ny;
  a.w = w;
  a.w_ld = dv;
  a.ta = alpha;
  a.ta_ld = dv;
  a.sigma = sigma < 1e-10 ? 1e-10 : sigma;
  a.out0 = o0;
  a.out0_ld = op_outputs(op, d, dv);
  a.out1 = o1;
  a.out1_ld = d;
  a.nsplit = 1;
  if (op == OP_GRADDIM) a.p0 = 0;
  if (op == OP_HESSRC) a.p0 = a.p1 = 0;
  return a;
}

int tune_checks(gbk_ctx *c, int op, int d, int dv, long nx, long ny) {
  if (op < 0 || op >= OP_COUNT || !tunable_op(op))
    return c->fail(GBK_ERR_ARG, "op %d cannot be tuned (Convolve, the gradients and the Hessians can)", op);
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "dimension %d", d);
  int cnt;
  const int *sup = supported_dv(d, &cnt);
  if (std::find(sup, sup + cnt, dv) == sup + cnt)
    return c->fail(GBK_ERR_UNSUPPORTED, "dv = %d is not a compiled column width (tune each column chunk)", dv);
  if (nx <= 0 || ny <= 0) return c->fail(GBK_ERR_ARG, "autotune needs nx, ny > 0");
  if (c->capturing()) return c->fail(GBK_ERR_STATE, "autotune during stream capture");
  if (cudaSetDevice(c->device) != cudaSuccess) return c->fail(GBK_ERR_CUDA, "cudaSetDevice");
  return GBK_OK;
}

}  // namespace

extern "C" {

int gbk_autotune(gbk_ctx *c, int op, int d, int dv, long nx, long ny, double sigma) {
  if (!c) return GBK_ERR_ARG;
  c->err.clear();
  ++c->call_epoch;
  if (int rc = tune_checks(c, op, d, dv, nx, ny)) return rc;
  TuneBuffers tb;
  const long nin = std::max(nx, ny);
  const size_t sz_x = (size_t)nin * d, sz_w = (size_t)nin * dv;
  double *X = tb.get(sz_x), *Y = tb.get(sz_x), *Wt = tb.get(sz_w), *A = tb.get(sz_w);
  double *O0 = tb.get((size_t)nx * op_outputs(op, d, dv)), *O1 = tb.get((size_t)nx * d);
  if (!X || !Y || !Wt || !A || !O0 || !O1) return c->fail(GBK_ERR_ALLOC, "autotune buffers");
  fill_uniform_kernel<<<(unsigned)((sz_x + 255) / 256), 256, 0, c->stream>>>(X, (long)sz_x, 1, 0.0, 1.0);
  fill_uniform_kernel<<<(unsigned)((sz_x + 255) / 256), 256, 0, c->stream>>>(Y, (long)sz_x, 2, 0.0, 1.0);
  fill_uniform_kernel<<<(unsigned)((sz_w + 255) / 256), 256, 0, c->stream>>>(Wt, (long)sz_w, 3, -1.0, 1.0);
  fill_uniform_kernel<<<(unsigned)((sz_w + 255) / 256), 256, 0, c->stream>>>(A, (long)sz_w, 4, -1.0, 1.0);
  if (int rc = c->cuda(cudaGetLastError(), "autotune inputs")) return rc;
  return tune_core(c, op, d, dv, tune_args(op, d, dv, X, nx, Y, Wt, ny, sigma, A, O0, O1), nullptr, nullptr, nullptr);
}

int gbk_autotune_data(gbk_ctx *c, int op, int d, int dv, const double *x, long nx, const double *y, const double *w,
                      long ny, double sigma, const double *alpha, int *variant, int *nsplit, double *ms) {
  if (!c) return GBK_ERR_ARG;
  c->err.clear();
  ++c->call_epoch;
  if (int rc = tune_checks(c, op, d, dv, nx, ny)) return rc;
  if (!x || !y || !w || ((op == OP_CONV_GRADA || op == OP_GRADA) && !alpha)) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  const double *da = alpha ? io.in(alpha, (size_t)nx * dv, "alpha") : nullptr;
  if (io.rc) return io.rc;
  TuneBuffers tb;
  double *O0 = tb.get((size_t)nx * op_outputs(op, d, dv)), *O1 = tb.get((size_t)nx * d);
  if (!O0 || !O1) return c->fail(GBK_ERR_ALLOC, "autotune buffers");
  float best_ms = 0.f;
  int rc = tune_core(c, op, d, dv, tune_args(op, d, dv, dx, nx, dy, dw, ny, sigma, da, O0, O1), variant, nsplit,
                     &best_ms);
  if (!rc && ms) *ms = best_ms;
  if (!rc) rc = io.finish();
  return rc;
}

int gbk_tune_save(const gbk_ctx *c, const char *path) {
  if (!c || !path) return GBK_ERR_ARG;
  FILE *f = fopen(path, "w");
  if (!f) return GBK_ERR_ARG;
  for (const auto &kv : c->tune) {
    int op, mode, d, dv, bx, by, path;
    std::tie(op, mode, d, dv, bx, by, path) = kv.first;
    fprintf(f,
            "{\"op\": %d, \"mode\": %d, \"d\": %d, \"dv\": %d, \"bx\": %d, \"by\": %d, \"path\": %d, "
            "\"variant\": %d, \"nsplit\": %d}\n",
            op, mode, d, dv, bx, by, path, kv.second.first, kv.second.second);
  }
  fclose(f);
  return GBK_OK;
}

int gbk_tune_load(gbk_ctx *c, const char *path) {
  if (!c || !path) return GBK_ERR_ARG;
  FILE *f = fopen(path, "r");
  if (!f) return c->fail(GBK_ERR_ARG, "cannot open %s", path);
  char line[512];
  int bad = 0;
  while (fgets(line, sizeof line, f)) {
    int op, mode, d, dv, bx, by, path, v, ns;
    if (sscanf(line,
               "{\"op\": %d, \"mode\": %d, \"d\": %d, \"dv\": %d, \"bx\": %d, \"by\": %d, \"path\": %d, "
               "\"variant\": %d, \"nsplit\": %d}",
               &op, &mode, &d, &dv, &bx, &by, &path, &v, &ns) != 9) {
      ++bad;
      continue;
    }
    KernelEntry e;
    // entries for variants this build does not compile, or malformed, are skipped
    if (op < 0 || op >= OP_COUNT || path < 0 || path > 2 || ns < 0 || !find_kernel(op, mode, d, dv, v, &e)) {
      ++bad;
      continue;
    }
    c->tune[gbk_ctx::TuneKey{op, mode, d, dv, bx, by, path}] = {v, ns};
  }
  (void)bad;
  fclose(f);
  return GBK_OK;
}

}  // extern "C"
