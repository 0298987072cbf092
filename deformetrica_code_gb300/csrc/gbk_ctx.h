// The context behind the opaque gbk_ctx handle of include/gbk.h.
//
// It replaces the legacy CUDA path's per-call cudaMalloc / cudaMemcpy / cudaFree
// (lib/cuda_convolutions/GpuConv1D.cu:97-130): device buffers live as long as the context and
// only grow, the stream is the caller's choice, and every CUDA status is checked.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <map>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "gbk_dispatch.h"

// A profiler range (NVTX) over the scope of one C ABI call, named after the call; inert unless a
// profiling tool is attached.
struct GbkRange {
  explicit GbkRange(const char *name) { nvtxRangePushA(name); }
  ~GbkRange() { nvtxRangePop(); }
  GbkRange(const GbkRange &) = delete;
  GbkRange &operator=(const GbkRange &) = delete;
};
#define GBK_RANGE() GbkRange gbk_nvtx_range_(__func__)

struct gbk_ctx {
  struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
  };
  static constexpr int kStageSlots = 12;

  int device = 0;
  int num_sms = 1;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  int mode = 0;         // GBK_MODE_F32C / GBK_MODE_F64
  int force_split = 0;  // 0 = automatic
  size_t alloc_limit = 0;  // fault injection: buffer growth beyond this fails (0 = none)
  int inject_pointer_device = -1;  // fault injection: device pointers reported on this GPU (-1 = none)
  long long launches = 0;
  std::string err;

  DevBuf partial;             // source-split partial sums
  DevBuf tickets;             // per target tile: split CTAs done (the fused split reduction)
  DevBuf stage[kStageSlots];  // host-argument staging
  DevBuf reduce;              // FP64 reductions and small temporaries
  DevBuf tmp;                 // op temporaries (e.g. K w for the kernel norm)
  DevBuf packed;              // packed coordinates of the small FP32 shapes (PairArgs::xp / yp)
  int order = 0;              // GBK_ORDER_* (0 = automatic)
  int gradient_mode = 0;      // GBK_GRADIENT_* of the point-cloud and volume data terms
  int estimator = 0;          // GBK_ESTIMATOR_* of the *_optimize calls
  struct SortSlot {           // a point set in spatial order: perm, sorted keys, box
    DevBuf buf;
    const double *ptr = nullptr;
    long n = 0;
    int d = 0;
    int key_bits = 0;
    long long epoch = -1;     // call_epoch of the sort
    long long last_use = 0;
  };
  SortSlot sort_slot[2];
  long long sort_clock = 0;
  long long call_epoch = 0;   // advanced by every API entry
  bool order_cache = false;   // reuse sorts within the current API call (inputs unchanged)
  DevBuf order_keep[2];       // target tiles / source chunk boxes of the last launch
  DevBuf order_tmp;           // Morton keys and block boxes
  DevBuf order_cub;           // radix-sort scratch
  DevBuf order_src;           // source rows in sorted order
  DevBuf order_box;           // the automatic order's extent box and its block partials
  double *host_box = nullptr; // pinned host copy of that box (allocated by gbk_create)
  struct AutoOrder {          // the automatic order's extent test for the point sets of this API call
    long long epoch = -1;
    const double *x = nullptr, *y = nullptr;
    long nx = 0, ny = 0;
    double sigma = 0.0;
    bool wide = false;        // spread wider than a cell of the spatial order
  } auto_order_cache;
  enum { AUTO_OFF = 0, AUTO_TWO_FLOAT = 1, AUTO_SPATIAL = 2 };
  // device, one allocation: [0] unused, [1] the spatial order's ticket, [2] the non-finite flag,
  // [3] the status word, [4 + op] pairs evaluated by the kernel sums of operation op
  unsigned long long *pair_counter = nullptr;
  static constexpr int kCounterWords = 4 + gbk::OP_COUNT;
  unsigned long long *pair_counter_of(int op) const { return pair_counter ? pair_counter + 4 + op : nullptr; }
  unsigned *order_ticket = nullptr;            // device: in the pair counter's allocation
  unsigned *nonfinite = nullptr;               // device: a pruned launch's targets hold a NaN or inf
  unsigned *status = nullptr;                  // device: bit 0 = a bounded wait gave up (gbk_synchronize)
  int staging = 0;                             // GBK_STAGING_* of the spatial order's source tiles
  int last_variant = -1, last_nsplit = 0;      // the last kernel-sum launch (gbk_last_launch)
  // GBK_STAGING_AUTO: the spatial order stages with bulk asynchronous copies. Measured on GB300, fused
  // Convolve + alpha-gradient pass, N = M = 1e6, d = 3, sorted: 531.5 ms against 548.1 ms with
  // ordinary loads at sigma = 0.1, 128.1 against 133.8 ms at sigma = 0.02; 5.92 against 6.07 ms at
  // N = M = 1e5 (bitwise identical results).
  static constexpr bool kBulkByDefault = true;

  // op, mode, d, dv, log2 nx, log2 ny, path (PATH_*)
  typedef std::tuple<int, int, int, int, int, int, int> TuneKey;
  std::map<TuneKey, std::pair<int, int>> tune;  // -> (variant, nsplit; nsplit 0 = the heuristic's)
  // The path of a kernel-sum launch: caller order with one-float or two-float coordinates, or the
  // spatial order. The tuning table is kept per path.
  enum { PATH_PLAIN = 0, PATH_TWO_FLOAT = 1, PATH_SPATIAL = 2 };
  struct LaunchPlan {
    int path = PATH_PLAIN;
    int variant = 0;
    bool spatial = false, prune = false;
  };
  // Shape variants 0 .. kNumShapeVariants - 1 (default, 2-way unroll, 4 targets per thread, scalar
  // lanes, 128-thread CTAs) where compiled (gbk_k_conv*.cu)
  static constexpr int kNumShapeVariants = 5;
  std::map<const void *, int> occ_cache;

  int fail(int code, const char *fmt, ...);
  int cuda(cudaError_t e, const char *what);
  bool capturing() const;
  int ensure(DevBuf &b, size_t bytes, const char *what);
  TuneKey key(int op, int d, int dv, long nx, long ny, int path) const;
  int plan(int op, int d, int dv, const gbk::PairArgs &a, LaunchPlan *p);
  std::vector<int> family(int path, int op, int d, int dv) const;
  int occupancy(const gbk::KernelEntry &e, int d);
  int choose_split(const gbk::KernelEntry &e, int d, long nx, long ny);
  int launch(int op, int d, int dv, gbk::PairArgs a);
  int ensure_tickets(long n);
  int auto_order(int op, int d, const gbk::PairArgs &a, int *choice);

  // Lets launches of one API call reuse spatial sorts of the same (unchanged) rows.
  struct OrderCacheScope {
    gbk_ctx *c;
    bool saved;
    OrderCacheScope(gbk_ctx *ctx) : c(ctx), saved(ctx->order_cache) { c->order_cache = true; }
    ~OrderCacheScope() { c->order_cache = saved; }
  };

  // Holds the order policy at `o` for a scope (the registration, atlas and regression steps use
  // TWO_FLOAT: caller order, adaptive two-float coordinates for the Convolve-like ops).
  struct OrderScope {
    gbk_ctx *c;
    int saved;
    OrderScope(gbk_ctx *ctx, int o) : c(ctx), saved(ctx->order) { c->order = o; }
    ~OrderScope() { c->order = saved; }
  };

  // the particle-mesh kernel's cached FFT plans and kernel spectra (gbk_p3m.cu)
  void *p3m = nullptr;
  void (*p3m_free)(void *) = nullptr;

  void release() {
    if (p3m && p3m_free) p3m_free(p3m);
    p3m = nullptr;
    auto fr = [](DevBuf &b) {
      if (b.p) cudaFree(b.p);
      b.p = nullptr;
      b.cap = 0;
    };
    fr(partial);
    fr(tickets);
    fr(reduce);
    fr(tmp);
    fr(packed);
    fr(order_keep[0]);
    fr(order_keep[1]);
    for (auto &ss : sort_slot) {
      fr(ss.buf);
      ss.ptr = nullptr;
      ss.epoch = -1;
    }
    fr(order_tmp);
    fr(order_cub);
    fr(order_src);
    fr(order_box);
    if (pair_counter) cudaFree(pair_counter);
    pair_counter = nullptr;
    order_ticket = nullptr;
    nonfinite = nullptr;
    status = nullptr;
    for (auto &b : stage) fr(b);
    if (host_box) cudaFreeHost(host_box);
    host_box = nullptr;
  }
};
