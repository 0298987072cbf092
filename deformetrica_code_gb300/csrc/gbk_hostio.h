// Host/device pointer handling of the C ABI: device pointers are used in place; host pointers
// are staged through the context's device buffers (inputs copied in before the kernels, outputs
// copied back and the stream synchronised at the end), which is the synchronous host-pointer
// behaviour of the reference's GaussGpu*Conv1D (lib/cuda_convolutions/GpuConv1D.cu:97-130).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"

inline bool is_device_pointer(const void *p) {
  if (!p) return true;
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// Stages host arguments through the context's device buffers.
struct HostIO {
  gbk_ctx *c;
  int slot = 0;
  int rc = GBK_OK;
  bool any_host = false;
  struct Out {
    double *host;
    double *dev;
    size_t n;
  };
  std::vector<Out> outs;
  explicit HostIO(gbk_ctx *ctx) : c(ctx) {}

  template <typename P>
  const P *in(const P *p, size_t n, const char *name) {
    if (rc || !p || n == 0 || is_device_pointer(p)) return p;
    any_host = true;
    if (slot >= gbk_ctx::kStageSlots) {
      rc = c->fail(GBK_ERR_ARG, "too many host arguments");
      return nullptr;
    }
    gbk_ctx::DevBuf &b = c->stage[slot++];
    rc = c->ensure(b, n * sizeof(P), name);
    if (rc) return nullptr;
    rc = c->cuda(cudaMemcpyAsync(b.p, p, n * sizeof(P), cudaMemcpyHostToDevice, c->stream),
                 "cudaMemcpyAsync H2D");
    return rc ? nullptr : (const P *)b.p;
  }
  double *out(double *p, size_t n, const char *name) {
    if (rc || !p || n == 0 || is_device_pointer(p)) return p;
    any_host = true;
    if (slot >= gbk_ctx::kStageSlots) {
      rc = c->fail(GBK_ERR_ARG, "too many host arguments");
      return nullptr;
    }
    gbk_ctx::DevBuf &b = c->stage[slot++];
    rc = c->ensure(b, n * sizeof(double), name);
    if (rc) return nullptr;
    outs.push_back({p, (double *)b.p, n});
    return (double *)b.p;
  }
  int finish() {
    if (rc) return rc;
    for (auto &o : outs) {
      rc = c->cuda(cudaMemcpyAsync(o.host, o.dev, o.n * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                   "cudaMemcpyAsync D2H");
      if (rc) return rc;
    }
    if (any_host) rc = c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize");
    return rc;
  }
};

