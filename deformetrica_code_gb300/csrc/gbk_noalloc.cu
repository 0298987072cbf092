// gbk_kernel_norm_noalloc: the RKHS norm <w, K w> for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at the moment they need this quantity: an optimiser loop
// running inside a memory budget fixed at start-up, code that only owns a pre-sized memory pool,
// or a stream whose every operation must be known in advance. gbk_kernel_norm itself grows the
// context's device buffers on first use (the K w intermediate and the source-split partials), so
// this variant keeps that scratch in one file-scope __device__ array instead, loaded with the
// library: every GPU that loads libgbkernel.so holds kNoAllocScratchDoubles doubles (16 MiB) of it
// until the process exits.
//
// Contract (also in include/gbk.h):
//  * inputs and the output are device pointers owned by the caller;
//  * n * dv must not exceed kNoAllocScratchDoubles (the K w intermediate); otherwise the call
//    returns GBK_ERR_ARG without launching anything;
//  * no cudaMalloc / cudaFree or other allocating routine is called;
//  * the first call on a device looks up the array's device address (cudaGetSymbolAddress with
//    that device current); make that first call before any stream capture: a first call made while
//    the context's stream is capturing returns GBK_ERR_STATE. gbk_create looks the address up again
//    for its device if it was cached, so contexts created after a cudaDeviceReset see the new one;
//  * device memory of another GPU than the context's is refused with GBK_ERR_ARG, as is a NaN
//    kernel width;
//  * all calls share the one array: calls that overlap on the GPU (two streams, two host threads)
//    race on it, so serialise them. Nothing in the array needs to start at zero: each call writes
//    every element it later reads.
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_dispatch.h"
#include "gbk_hostio.h"
#include "gbk_ops.h"

namespace {

constexpr size_t kNoAllocScratchDoubles = (size_t)2 << 20;  // 2 Mi doubles = 16 MiB per device
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

std::mutex g_setup_mutex;
double *g_scratch_addr[kMaxDevices] = {nullptr};

// Device address of the scratch array for `device` (current); looked up once per device. The first
// lookup may load the module holding the array, which must not happen inside a stream capture.
int scratch_address(gbk_ctx *c, double **out) {
  const int device = c->device;
  if (device < 0 || device >= kMaxDevices)
    return c->fail(GBK_ERR_UNSUPPORTED, "allocation-free kernel norm: device %d above %d", device, kMaxDevices - 1);
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) {
    if (c->capturing())
      return c->fail(GBK_ERR_STATE, "allocation-free kernel norm: the first call on GPU %d must come before "
                     "stream capture (it looks up the scratch array's address)", device);
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return c->fail(GBK_ERR_CUDA, "cudaGetSymbolAddress of the scratch array: %s", cudaGetErrorString(e));
    }
    g_scratch_addr[device] = static_cast<double *>(p);
  }
  *out = g_scratch_addr[device];
  return GBK_OK;
}

}  // namespace

namespace gbk {
// Called by gbk_create with `device` current: a cached address is looked up again, so a context
// created after cudaDeviceReset (which unloads the module holding the array) gets the new one.
void noalloc_refresh_device(int device) {
  if (device < 0 || device >= kMaxDevices) return;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_addr[device]) return;
  void *p = nullptr;
  if (cudaGetSymbolAddress(&p, g_noalloc_scratch) == cudaSuccess && p)
    g_scratch_addr[device] = static_cast<double *>(p);
  else
    g_scratch_addr[device] = nullptr;
  cudaGetLastError();
}
}  // namespace gbk

extern "C" int gbk_kernel_norm_noalloc(gbk_ctx *c, int d, int dv, const double *y, const double *w,
                                       long n, double sigma, double *out) {
  using namespace gbk;
  if (!c) return GBK_ERR_ARG;
  c->err.clear();
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "dimension %d not supported (2 or 3)", d);
  if (dv <= 0 || n <= 0) return c->fail(GBK_ERR_ARG, "needs n > 0 points and dv > 0 weight columns");
  if (!y || !w || !out) return c->fail(GBK_ERR_ARG, "null pointer");
  if (!(sigma == sigma)) return c->fail(GBK_ERR_ARG, "kernel width is NaN");
  if ((size_t)n * (size_t)dv > kNoAllocScratchDoubles)
    return c->fail(GBK_ERR_ARG, "n * dv = %zu is above the scratch capacity of %zu doubles", (size_t)n * dv,
                   kNoAllocScratchDoubles);
  if (cudaSetDevice(c->device) != cudaSuccess) {
    cudaGetLastError();
    return c->fail(GBK_ERR_CUDA, "cudaSetDevice(%d)", c->device);
  }
  const void *args[3] = {y, w, out};
  const char *names[3] = {"y", "w", "out"};
  for (int k = 0; k < 3; ++k) {  // device memory of the context's GPU only; nothing is staged
    bool dev = false;
    if (int rc = locate(c, args[k], names[k], &dev)) return rc;
    if (!dev) return c->fail(GBK_ERR_ARG, "%s: host memory (this entry point takes device pointers only)", names[k]);
  }
  double *scratch = nullptr;
  if (int rc = scratch_address(c, &scratch)) return rc;

  // scratch = [K w : n x dv][split partials : nsplit x chunk width x n]
  double *kw = scratch;
  const size_t free_doubles = kNoAllocScratchDoubles - (size_t)n * dv;
  int cnt;
  const int *sup = supported_dv(d, &cnt);
  for (int c0 = 0, rem = dv; rem > 0;) {
    int cw = 0;
    for (int k = 0; k < cnt; ++k)
      if (sup[k] <= rem) {
        cw = sup[k];
        break;
      }
    KernelEntry e;
    if (!find_kernel(OP_CONV, c->mode, d, cw, 0, &e)) return c->fail(GBK_ERR_UNSUPPORTED, "no kernel for dv = %d", cw);
    // source splits: enough CTAs for every SM, at most what the free scratch holds
    int occ = 1;
    if (e.smem > 48 * 1024 &&  // as the launch itself will: the occupancy query needs it first
        cudaFuncSetAttribute(e.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, e.smem) != cudaSuccess)
      cudaGetLastError();
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, e.kernel, e.block, e.smem) != cudaSuccess || occ < 1) {
      cudaGetLastError();
      occ = 1;
    }
    const long per_cta = (long)e.block * e.r;
    const long itiles = (n + per_cta - 1) / per_cta;
    long want = std::max(1L, ((long)c->num_sms * occ + itiles - 1) / itiles);
    want = std::min(want, std::max(1L, n / (2L * e.tj)));
    const long fit = (long)(free_doubles / ((size_t)e.no * n));
    const int ns = (int)std::max(1L, std::min(want, fit));
    PairArgs a = pair_args(n, n, sigma);
    a.x = y;
    a.y = y;
    a.w = w + c0;
    a.w_ld = dv;
    a.out0 = kw + c0;
    a.out0_ld = dv;
    a.partial = ns > 1 ? kw + (size_t)n * dv : nullptr;
    if (int rc = c->cuda(e.fn(a, ns, c->stream), "kernel launch")) return rc;
    c->launches += ns > 1 ? 2 : 1;
    c0 += cw;
    rem -= cw;
  }
  if (int rc = c->cuda(dot_f64(c->stream, w, kw, n * (long)dv, out, 0), "FP64 dot")) return rc;
  c->launches += 1;
  return GBK_OK;
}
