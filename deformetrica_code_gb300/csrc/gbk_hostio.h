// Host/device pointer handling of the C ABI: device pointers are used in place; host pointers
// are staged through the context's device buffers (inputs copied in before the kernels, outputs
// copied back and the stream synchronised at the end), which is the synchronous host-pointer
// behaviour of the reference's GaussGpu*Conv1D (lib/cuda_convolutions/GpuConv1D.cu:97-130).
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"

// Where a pointer lives for a context on GPU `device`: kHostMemory (staged through the context's
// buffers), kThisDevice (device memory of that GPU, or managed memory) or kOtherDevice (device
// memory of another GPU: the kernels cannot read it without peer access, so the call refuses it).
// `injected` >= 0 reports every device allocation as memory of that GPU (fault injection, so the
// other-GPU refusal can be tested with one GPU).
enum PointerHome { kHostMemory = 0, kThisDevice = 1, kOtherDevice = 2 };

inline PointerHome pointer_home(const void *p, int device, int injected) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return kHostMemory;
  }
  if (at.type == cudaMemoryTypeManaged) return kThisDevice;
  if (at.type != cudaMemoryTypeDevice) return kHostMemory;
  const int home = injected >= 0 ? injected : at.device;
  return home == device ? kThisDevice : kOtherDevice;
}

// Whether p is usable in place by the context's kernels (*dev), refusing device memory of
// another GPU with GBK_ERR_ARG.
inline int locate(gbk_ctx *c, const void *p, const char *name, bool *dev) {
  const PointerHome h = pointer_home(p, c->device, c->inject_pointer_device);
  *dev = h == kThisDevice;
  if (h == kOtherDevice)
    return c->fail(GBK_ERR_ARG, "%s: device memory of another GPU than the context's GPU %d", name, c->device);
  return GBK_OK;
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

  // Device memory of another GPU is refused with GBK_ERR_ARG before anything is queued.
  bool device_resident(const void *p, const char *name) {
    const PointerHome h = pointer_home(p, c->device, c->inject_pointer_device);
    if (h == kOtherDevice) {
      rc = c->fail(GBK_ERR_ARG, "%s: device memory of another GPU than the context's GPU %d", name, c->device);
      return true;
    }
    return h == kThisDevice;
  }

  template <typename P>
  const P *in(const P *p, size_t n, const char *name) {
    if (rc || !p || n == 0) return p;
    if (device_resident(p, name)) return rc ? nullptr : p;
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
    if (rc || !p || n == 0) return p;
    if (device_resident(p, name)) return rc ? nullptr : p;
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

