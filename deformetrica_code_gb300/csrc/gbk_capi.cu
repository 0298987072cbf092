// C ABI of libgbkernel.so: contexts, argument checks, host/device pointer staging, column
// chunking, the source-split heuristic and the autotuner. The entry points are declared (with
// the reference method each replaces) in include/gbk.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/gbk.h"
#include "gbk_ctx.h"
#include "gbk_dispatch.h"
#include "gbk_hostio.h"
#include "gbk_order.h"

using namespace gbk;

// =============================================================================================
// kernel table
// =============================================================================================
namespace gbk {

int op_outputs(int op, int d, int dv) {
  switch (op) {
    case OP_CONV: return dv;
    case OP_CONV_GRADA: return dv + d;
    case OP_GRADA: return d;
    case OP_VARLIN: return dv * d;
    case OP_GRADDIM: return dv;
    case OP_HESSFULL: return dv * (d * (d + 1) / 2 + 1);
    case OP_HESSRC: return 2 * dv;
    case OP_SPECIAL: return 2 * d;
    case OP_ADJCP: return 5 * d;
  }
  return 0;
}

bool find_kernel(int op, int mode, int d, int dv, int variant, KernelEntry *e) {
  if (variant == VARIANT_TWO_FLOAT || variant == VARIANT_SMALL_TWO_FLOAT)  // Convolve-like ops only
    return (op == OP_CONV || op == OP_CONV_GRADA || op == OP_GRADA) && find_kernel_conv(op, mode, d, dv, variant, e);
  if (variant == VARIANT_BULK || variant == VARIANT_BULK_128)
    return mode == MODE_F32C && find_kernel_conv_bulk(op, d, dv, variant, e);
  if (variant == VARIANT_WARP || variant == VARIANT_WARP_TWO_FLOAT)
    return mode == MODE_F32C && find_kernel_warp(op, d, dv, variant, e);
  switch (op) {
    case OP_CONV:
    case OP_CONV_GRADA:
    case OP_GRADA: return find_kernel_conv(op, mode, d, dv, variant, e);
    case OP_VARLIN:
    case OP_GRADDIM: return find_kernel_grad(op, mode, d, dv, variant, e);
    case OP_HESSFULL:
    case OP_HESSRC:
    case OP_SPECIAL: return find_kernel_hess(op, mode, d, dv, variant, e);
    case OP_ADJCP: return find_kernel_deform(op, mode, d, dv, variant, e);
  }
  return false;
}

const int *supported_dv(int d, int *count) {
  static const int dv2[] = {4, 3, 2, 1};
  static const int dv3[] = {6, 3, 2, 1};
  *count = 4;
  return d == 2 ? dv2 : dv3;
}

}  // namespace gbk

// =============================================================================================
// context helpers
// =============================================================================================
int gbk_ctx::fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  err = buf;
  return code;
}

int gbk_ctx::cuda(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return GBK_OK;
  cudaGetLastError();
  return fail(e == cudaErrorMemoryAllocation ? GBK_ERR_ALLOC : GBK_ERR_CUDA, "%s: %s", what,
              cudaGetErrorString(e));
}

bool gbk_ctx::capturing() const {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(stream, &st) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return st != cudaStreamCaptureStatusNone;
}

int gbk_ctx::ensure(DevBuf &b, size_t bytes, const char *what) {
  if (b.cap >= bytes) return GBK_OK;
  if (capturing())
    return fail(GBK_ERR_STATE, "%s: needs %zu bytes of device scratch while the stream is being captured; "
                "run the call once before capture", what, bytes);
  if (alloc_limit && bytes > alloc_limit)
    return fail(GBK_ERR_ALLOC, "%s: %zu bytes refused (injected allocation limit %zu)", what, bytes, alloc_limit);
  if (b.p) {
    int rc = cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
    if (rc) return rc;
    cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
  }
  size_t want = std::max(bytes, b.cap + b.cap / 2);
  want = (want + 255) & ~(size_t)255;
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    e = cudaMalloc(&p, bytes);
    want = bytes;
  }
  if (e != cudaSuccess) return cuda(e, what);
  b.p = p;
  b.cap = want;
  return GBK_OK;
}

// Zeroed counters for `n` target tiles (grow-only; the kernels reset every counter they use).
int gbk_ctx::ensure_tickets(long n) {
  const size_t bytes = (size_t)std::max(n, 1L) * sizeof(unsigned);
  if (tickets.cap >= bytes) return GBK_OK;
  if (int rc = ensure(tickets, bytes, "split tickets")) return rc;
  return cuda(cudaMemsetAsync(tickets.p, 0, tickets.cap, stream), "ticket reset");
}

// Tuning-table key: operation, precision, shape and size buckets (powers of two).
static int bucket(long n) {
  int b = 0;
  while (n > 1) {
    n >>= 1;
    ++b;
  }
  return b;
}

gbk_ctx::TuneKey gbk_ctx::key(int op, int d, int dv, long nx, long ny, int path) const {
  return TuneKey{op, mode, d, dv, bucket(nx), bucket(ny), path};
}

int gbk_ctx::occupancy(const KernelEntry &e, int) {
  auto it = occ_cache.find(e.kernel);
  if (it != occ_cache.end()) return it->second;
  int blocks = 0;
  if (e.smem > 48 * 1024)
    cudaFuncSetAttribute(e.kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, e.smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, e.kernel, e.block, e.smem) != cudaSuccess)
    blocks = 1;
  cudaGetLastError();
  if (blocks < 1) blocks = 1;
  occ_cache[e.kernel] = blocks;
  return blocks;
}

// Source splits: enough CTAs to fill every SM with a small tail, each split >= 2 source tiles. A
// warp-split kernel (e.ks > 0) aims at two CTAs per SM, each of its warps keeping >= one tile.
int gbk_ctx::choose_split(const KernelEntry &e, int d, long nx, long ny) {
  if (force_split > 0) return force_split;
  if (e.ks > 0) {
    const long itiles = std::max(1L, (nx + e.tile - 1) / e.tile);
    long cap = std::max(1L, ny / ((long)e.ks * e.tj));
    cap = std::min(cap, 64L);
    cap = std::min(cap, std::max(1L, (long)((512L << 20) / (8L * e.no * std::max(nx, 1L)))));
    return (int)std::max(1L, std::min(cap, (2L * num_sms + itiles - 1) / itiles));
  }
  long per_cta = (long)e.tile;
  long itiles = (nx + per_cta - 1) / per_cta;
  long slots = (long)num_sms * occupancy(e, d);
  long max_split = std::max(1L, ny / (2L * e.tj));
  max_split = std::min(max_split, 64L);
  // partial buffer limit: 512 MiB
  long cap = std::max(1L, (long)((512L << 20) / (8L * e.no * std::max(nx, 1L))));
  max_split = std::min(max_split, cap);
  double best = 1e300;
  int best_s = 1;
  for (long s = 1; s <= max_split; ++s) {
    long ctas = itiles * s;
    double waves = std::ceil((double)ctas / (double)slots);
    double t = waves / (double)s + 0.002 * s;  // per-CTA work ~ 1/s, small per-split overhead
    if (t < best - 1e-9) {
      best = t;
      best_s = (int)s;
    }
  }
  return best_s;
}

// GBK_ORDER_AUTO: caller order (AUTO_OFF), caller order with adaptive two-float coordinates
// (AUTO_TWO_FLOAT) or the spatial order (AUTO_SPATIAL).
//  * Large calls (nx, ny >= 4096 and nx ny >= 2^30) are always ordered: the sort costs about 1 %
//    there when it does not help, and pruning and accuracy gain when it does.
//  * Below that, in FP32C mode, Convolve, the alpha-gradient and their fusion run their adaptive
//    two-float variant in caller order: each CTA whose targets spread wider than kTwoFloatWidth
//    scaled units forms its differences from hi + lo coordinates, every other CTA runs the one-float
//    loop, so accuracy no longer depends on the spread and narrow data pays nothing.
//  * Other ops of at least kAutoMinPairs pairs measure the largest extent of the union of the two
//    point sets in units of the FP32 coordinate scale (sqrt(log2 e) / sigma per input unit) and take
//    the spatial order above kAutoCellWidth: in caller order a CTA's targets span the whole set, and
//    rounding the centred coordinates costs ~u (|x| + |y|) on every difference, while the order's
//    tiles are no wider than a cell of that width. The extent costs one small launch and one wait
//    for the stream, so it is skipped while the stream is being captured; within one API call the
//    decision for the same two point sets is reused.
//  * Smaller calls and FP64 calls (no centring) follow the size rule alone.
int gbk_ctx::auto_order(int op, int d, const PairArgs &a, int *choice) {
  constexpr double kAutoMinPairs = (double)(1L << 22);
  constexpr double kAutoCellWidth = 16.0;
  const double pairs = (double)a.nx * (double)a.ny;
  *choice = AUTO_OFF;
  if (a.nx >= 4096 && a.ny >= 4096 && pairs >= (double)(1L << 30)) {
    *choice = AUTO_SPATIAL;
    return GBK_OK;
  }
  if (mode != GBK_MODE_F32C) return GBK_OK;
  if (op == OP_CONV || op == OP_CONV_GRADA || op == OP_GRADA) {
    *choice = AUTO_TWO_FLOAT;
    return GBK_OK;
  }
  if (pairs < kAutoMinPairs || capturing()) return GBK_OK;
  AutoOrder &m = auto_order_cache;
  const bool same = m.epoch == call_epoch && m.sigma == a.sigma &&
                    ((m.x == a.x && m.nx == a.nx && m.y == a.y && m.ny == a.ny) ||
                     (m.x == a.y && m.nx == a.ny && m.y == a.x && m.ny == a.nx));
  if (!same) {
    double extent = 0.0;
    if (int rc = order_extent(this, d, a.x, a.nx, a.y, a.ny, &extent)) return rc;
    m.epoch = call_epoch;
    m.x = a.x;
    m.nx = a.nx;
    m.y = a.y;
    m.ny = a.ny;
    m.sigma = a.sigma;
    m.wide = !(extent * coord_scale<float>(a.sigma) <= kAutoCellWidth);  // NaN/inf extent: wide
  }
  if (m.wide) *choice = AUTO_SPATIAL;
  return GBK_OK;
}

// The path a kernel-sum launch takes and its default launch shape: the order (caller order, or the
// spatial order with or without pruning), the coordinate form (two-float variants in caller order
// below the size rule) and the staging (bulk copies in the spatial order), then the small shape
// when the default one cannot fill the GPU. Waits for the stream only where the automatic order
// measures the point sets' extent (gbk_ctx::auto_order).
int gbk_ctx::plan(int op, int d, int dv, const PairArgs &a, LaunchPlan *p) {
  *p = LaunchPlan();
  const bool unordered = !a.xperm && !a.xtiles && a.nx > 0 && a.ny > 0 && a.nx < INT_MAX && a.ny < INT_MAX;
  int choice = AUTO_OFF;
  if (unordered && order == GBK_ORDER_AUTO)
    if (int rc = auto_order(op, d, a, &choice)) return rc;
  if (unordered && order == GBK_ORDER_TWO_FLOAT && mode == GBK_MODE_F32C) choice = AUTO_TWO_FLOAT;
  KernelEntry et;
  if (choice == AUTO_TWO_FLOAT && !find_kernel(op, mode, d, dv, VARIANT_TWO_FLOAT, &et))
    choice = order == GBK_ORDER_AUTO ? AUTO_SPATIAL : AUTO_OFF;  // no two-float variant for this op
  if (unordered) {
    switch (order) {
      case GBK_ORDER_SPATIAL: p->spatial = p->prune = true; break;
      case GBK_ORDER_SPATIAL_NOPRUNE: p->spatial = true; break;
      case GBK_ORDER_AUTO: p->spatial = p->prune = choice == AUTO_SPATIAL; break;
      default: break;
    }
  }
  p->path = p->spatial ? PATH_SPATIAL : (choice == AUTO_TWO_FLOAT ? PATH_TWO_FLOAT : PATH_PLAIN);
  // Too little work for the default shape to fill the GPU (e.g. control points x control points):
  // the small shape (fewer targets per CTA, shorter source tiles, more splits).
  bool small = false;
  KernelEntry e0, es;
  if (find_kernel(op, mode, d, dv, 0, &e0)) {
    const long per_cta = (long)e0.tile;
    const long itiles = (a.nx + per_cta - 1) / per_cta;
    const long max_split = std::max(1L, a.ny / (2L * e0.tj));
    small = itiles * max_split < 2L * num_sms && find_kernel(op, mode, d, dv, VARIANT_SMALL, &es);
  }
  // too small for the default shape, in caller order: the warp-split kernel where it is compiled
  KernelEntry ew;
  const bool warp = small && !p->spatial && unordered && mode == MODE_F32C &&
                    find_kernel(op, mode, d, dv, p->path == PATH_TWO_FLOAT ? VARIANT_WARP_TWO_FLOAT : VARIANT_WARP,
                                &ew);
  if (warp) {
    p->variant = p->path == PATH_TWO_FLOAT ? VARIANT_WARP_TWO_FLOAT : VARIANT_WARP;
  } else if (p->path == PATH_TWO_FLOAT) {
    p->variant = small ? VARIANT_SMALL_TWO_FLOAT : VARIANT_TWO_FLOAT;
  } else {
    p->variant = small ? VARIANT_SMALL : 0;
    KernelEntry eb;
    if (p->spatial && !small && (staging == GBK_STAGING_BULK || (staging == GBK_STAGING_AUTO && kBulkByDefault)) &&
        find_kernel(op, mode, d, dv, VARIANT_BULK, &eb))
      p->variant = VARIANT_BULK;
  }
  return GBK_OK;
}

// Compiled variants a launch on `path` may take: the same arithmetic as the path's default, so a
// tuned choice never changes the accuracy (two-float variants stay two-float), and bulk staging only
// where the sources are the spatial order's copies (and the staging policy allows it).
std::vector<int> gbk_ctx::family(int path, int op, int d, int dv) const {
  std::vector<int> cand;
  if (path == PATH_TWO_FLOAT) {
    cand = {VARIANT_TWO_FLOAT, VARIANT_SMALL_TWO_FLOAT, VARIANT_WARP_TWO_FLOAT};
  } else {
    if (path == PATH_SPATIAL && staging != GBK_STAGING_LOADS) {
      cand.push_back(VARIANT_BULK);
      cand.push_back(VARIANT_BULK_128);
    }
    for (int v = 0; v < kNumShapeVariants; ++v) cand.push_back(v);
    cand.push_back(VARIANT_SMALL);
    if (path == PATH_PLAIN) cand.push_back(VARIANT_WARP);  // caller order only (packed coordinates)
  }
  std::vector<int> out;
  KernelEntry e;
  for (int v : cand)
    if (find_kernel(op, mode, d, dv, v, &e)) out.push_back(v);
  return out;
}

// Packed coordinates for the small FP32 shapes (PairArgs::xp / yp): per coordinate of x (the first
// nxd values) and y, the float pair (hi, lo) of v * s with hi = fl32(v s) and lo = fl32(v s - hi), lo = 0
// where hi is not finite (so an infinite coordinate stays infinite, as when the kernel converts it).
__global__ void pack_scaled_kernel(const double *x, long nxd, const double *y, long nyd, double s, float2 *xp,
                                   float2 *yp) {
  pdl_entry();
  for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nxd + nyd; k += (long)gridDim.x * blockDim.x) {
    const double v = (k < nxd ? x[k] : y[k - nxd]) * s;
    const float hi = (float)v;
    const float lo = isfinite(hi) ? (float)(v - (double)hi) : 0.f;
    if (k < nxd)
      xp[k] = make_float2(hi, lo);
    else
      yp[k - nxd] = make_float2(hi, lo);
  }
}

int gbk_ctx::launch(int op, int d, int dv, PairArgs a) {
  LaunchPlan pl;
  if (int rc = plan(op, d, dv, a, &pl)) return rc;
  long ticket_tiles = 0;  // target tiles of the launch (the fused split reduction's tickets)
  int variant = pl.variant, ns = 0;
  const bool spatial = pl.spatial, prune = pl.prune;
  auto it = tune.find(key(op, d, dv, a.nx, a.ny, pl.path));
  if (it != tune.end()) {
    const std::vector<int> fam = family(pl.path, op, d, dv);
    if (std::find(fam.begin(), fam.end(), it->second.first) != fam.end()) {
      variant = it->second.first;
      ns = it->second.second;
    }
  }
  KernelEntry e;
  if (!find_kernel(op, mode, d, dv, variant, &e) && !find_kernel(op, mode, d, dv, 0, &e))
    return fail(GBK_ERR_UNSUPPORTED, "no kernel for op %d, d=%d, dv=%d", op, d, dv);
  // packed coordinates need caller order and points on both sides; a warp-split kernel needs them
  const bool can_pack = !spatial && !a.xperm && !a.yperm && !a.xtiles && a.nx > 0 && a.ny > 0 && mode == MODE_F32C;
  if (e.ks > 0 && !can_pack) {
    variant = find_kernel(op, mode, d, dv, VARIANT_SMALL, &e) ? VARIANT_SMALL : 0;
    if (variant == 0 && !find_kernel(op, mode, d, dv, 0, &e))
      return fail(GBK_ERR_UNSUPPORTED, "no kernel for op %d, d=%d, dv=%d", op, d, dv);
    ns = 0;
  }
  if (force_split > 0) ns = force_split;
  if (ns <= 0) ns = choose_split(e, d, a.nx, a.ny);
  if (spatial) {
    // sorted copies of the source rows the op reads (y, the weight columns, the special Hessian's
    // xi); OpAdjointCP's source extras share arrays with its targets, so it gathers while staging
    SourceCopies want;
    if (op == OP_ADJCP) {  // p, xi_pos, xi_mom of the sources, read through the permutation
      const double *ex[3] = {a.w, a.tb, a.sb};
      for (int k = 0; k < 3; ++k) {
        want.chk[k] = ex[k];
        want.chk_ld[k] = want.chk_cols[k] = d;
      }
    } else {
      want.na = op == OP_SPECIAL ? 3 : 2;
      want.src[0] = a.y;
      want.ld[0] = want.cols[0] = d;
      want.src[1] = a.w;
      want.ld[1] = a.w_ld;
      want.cols[1] = op == OP_SPECIAL ? d : dv;
      want.src[2] = a.sb;
      want.ld[2] = a.sb_ld;
      want.cols[2] = d;
    }
    SortedSet xs, ys;
    OrderView tv, sv;
    if (int rc = order_sort(this, d, a.x, a.nx, &xs)) return rc;
    if (int rc = order_sort(this, d, a.y, a.ny, &ys)) return rc;
    if (int rc = order_targets(this, d, xs, e.tile, a.sigma, &tv)) return rc;
    if (int rc = order_sources(this, d, a.y, ys, e.tj, want, &sv)) return rc;
    launches += xs.launches + ys.launches;
    a.xperm = tv.perm;
    a.xtiles = tv.tiles;
    a.nxtiles = tv.ntiles;
    a.xtile_bound = tv.grid;
    ticket_tiles = tv.tile_bound;
    a.ybox = prune ? sv.boxes : nullptr;
    if (prune) {
      // the reference's sums are NaN or infinite wherever a target coordinate or extra is, however
      // small its kernel values: such a launch visits every chunk (source chunks holding a
      // non-finite value are never pruned either, see order_sources)
      const bool adj = op == OP_ADJCP;
      if (int rc = cuda(unbound_boxes_if_nonfinite(stream, d, a.x, a.nx, a.ta, a.ta_ld, a.tb, a.tb_ld,
                                                   adj ? a.sb : nullptr, adj ? a.sb_ld : 0, nonfinite,
                                                   const_cast<double *>(sv.boxes), (a.ny + e.tj - 1) / e.tj),
                        "non-finite check"))
        return rc;
      launches += 2;
    }
    launches += tv.launches + sv.launches;
    if (op == OP_ADJCP) {
      a.yperm = sv.perm;
    } else {
      a.y = sv.copies[0];
      a.w = sv.copies[1];
      a.w_ld = want.cols[1];
      if (op == OP_SPECIAL) {
        a.sb = sv.copies[2];
        a.sb_ld = d;
      }
    }
  }
  if (e.packable && can_pack) {
    // the small shapes centre in FP32 from coordinates packed once per launch (see packable)
    const bool same = a.x == a.y && a.nx == a.ny;
    const long nxd = a.nx * d, nyd = same ? 0 : a.ny * d;
    if (int rc = ensure(packed, (size_t)(nxd + nyd) * sizeof(float2), "packed coordinates")) return rc;
    float2 *xp = (float2 *)packed.p;
    const long tot = nxd + nyd;
    const unsigned blocks = (unsigned)std::min<long>((tot + 255) / 256, 4L * num_sms);
    if (int rc = cuda(gbk::launch(pack_scaled_kernel, blocks, 256, 0, stream, a.x, nxd, a.y, nyd,
                                  coord_scale<float>(a.sigma), xp, same ? xp : xp + nxd),
                      "coordinate packing"))
      return rc;
    launches += 1;
    a.xp = xp;
    a.yp = same ? xp : xp + nxd;
  }
  a.pair_count = pair_counter_of(op);
  a.status = status;
  // the bulk copies read whole chunks of the sorted copies, which order_sources pads to whole chunks
  a.bulk = spatial && (variant == VARIANT_BULK || variant == VARIANT_BULK_128) && op != OP_ADJCP && op != OP_SPECIAL && a.w_ld == dv ? 1 : 0;
  last_variant = variant;
  last_nsplit = ns;
  if (ns > 1) {
    // launch_pairs rounds the split count; size the buffer for the requested count
    int rc = ensure(partial, (size_t)ns * e.no * std::max(a.nx, 1L) * sizeof(double), "split partials");
    if (rc) return rc;
    a.partial = (double *)partial.p;
    // the last split CTA of each target tile reduces the tile (no separate reduction launch)
    if (!spatial) ticket_tiles = (a.nx + (long)e.tile - 1) / (long)e.tile;
    if ((rc = ensure_tickets(ticket_tiles))) return rc;
    a.tickets = (unsigned *)tickets.p;
  }
  int rc = cuda(e.fn(a, ns, stream), "kernel launch");
  if (rc) return rc;
  launches += 1;
  return GBK_OK;
}

// Splits dv weight columns into compiled chunk widths (largest first).
static std::vector<std::pair<int, int>> column_chunks(int d, int dv) {
  int cnt;
  const int *sup = supported_dv(d, &cnt);
  std::vector<std::pair<int, int>> ch;
  int c0 = 0, rem = dv;
  while (rem > 0) {
    for (int k = 0; k < cnt; ++k)
      if (sup[k] <= rem) {
        ch.push_back({c0, sup[k]});
        c0 += sup[k];
        rem -= sup[k];
        break;
      }
  }
  return ch;
}

static double clamp_sigma(double s) { return s < 1e-10 ? 1e-10 : s; }  // AbstractKernel.h:87-89

#define GBK_GUARD(ctx)                                                     \
  do {                                                                     \
    if (!(ctx)) return GBK_ERR_ARG;                                        \
    (ctx)->err.clear();                                                    \
    ++(ctx)->call_epoch;                                                   \
    if (cudaSetDevice((ctx)->device) != cudaSuccess) {                     \
      cudaGetLastError();                                                  \
      return (ctx)->fail(GBK_ERR_CUDA, "cudaSetDevice(%d)", (ctx)->device); \
    }                                                                      \
  } while (0)

static int check_common(gbk_ctx *c, int d, int dv, long nx, long ny, double sigma) {
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "dimension %d not supported (2 or 3)", d);
  if (dv <= 0) return c->fail(GBK_ERR_ARG, "weights need at least one column (dv=%d)", dv);
  if (nx < 0 || ny < 0) return c->fail(GBK_ERR_ARG, "negative row count");
  if (!(sigma == sigma)) return c->fail(GBK_ERR_ARG, "kernel width is NaN");
  if (nx > (1L << 31) || ny > (1L << 31)) return c->fail(GBK_ERR_ARG, "row count above 2^31");
  return GBK_OK;
}

static PairArgs base_args(long nx, long ny, double sigma) {
  PairArgs a;
  memset(&a, 0, sizeof a);
  a.nx = nx;
  a.ny = ny;
  a.sigma = clamp_sigma(sigma);
  a.nsplit = 1;
  return a;
}

// Runs a weight-linear op over column chunks. out0 per-column stride `ocol` (elements per weight
// column in one output row) and row stride dv*ocol; out1 (gradient) accumulates over chunks.
static int run_chunked(gbk_ctx *c, int op, int d, int dv, PairArgs a, const double *w,
                       const double *alpha, double *out0, int ocol, double *out1) {
  gbk_ctx::OrderCacheScope cache(c);  // the chunks share x and y
  auto ch = column_chunks(d, dv);
  for (size_t q = 0; q < ch.size(); ++q) {
    int c0 = ch[q].first, cw = ch[q].second;
    PairArgs b = a;
    b.w = w + c0;
    b.w_ld = dv;
    if (alpha) {
      b.ta = alpha + c0;
      b.ta_ld = dv;
    }
    b.out0 = out0 ? out0 + (long)c0 * ocol : nullptr;
    b.out0_ld = dv * ocol;
    b.out1 = out1;
    b.out1_ld = d;
    b.acc0 = 0;
    b.acc1 = q > 0 ? 1 : 0;
    int rc = c->launch(op, d, cw, b);
    if (rc) return rc;
  }
  return GBK_OK;
}

// =============================================================================================
// entry points
// =============================================================================================
extern "C" {

int gbk_version(void) { return 10000; }

static thread_local std::string g_create_err;

int gbk_create(int device, gbk_ctx **out) {
  if (!out) return GBK_ERR_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || device < 0 || device >= n) {
    cudaGetLastError();
    g_create_err = "no CUDA device " + std::to_string(device);
    return GBK_ERR_CUDA;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    cudaGetLastError();
    return GBK_ERR_CUDA;
  }
  gbk_ctx *c = new gbk_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    cudaGetLastError();
    delete c;
    return GBK_ERR_CUDA;
  }
  c->stream = c->own_stream;
  // pair counter and the spatial order's self-resetting ticket
  if (cudaMalloc(&c->pair_counter, gbk_ctx::kCounterWords * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMemset(c->pair_counter, 0, gbk_ctx::kCounterWords * sizeof(unsigned long long)) != cudaSuccess) {
    cudaGetLastError();
    c->release();
    cudaStreamDestroy(c->own_stream);
    delete c;
    g_create_err = "device allocation of the pair counter failed";
    return GBK_ERR_ALLOC;
  }
  if (cudaHostAlloc((void **)&c->host_box, 8 * sizeof(double), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    c->release();
    cudaStreamDestroy(c->own_stream);
    delete c;
    g_create_err = "pinned host allocation of the extent read-back failed";
    return GBK_ERR_ALLOC;
  }
  c->order_ticket = reinterpret_cast<unsigned *>(c->pair_counter + 1);
  c->nonfinite = reinterpret_cast<unsigned *>(c->pair_counter + 2);
  c->status = reinterpret_cast<unsigned *>(c->pair_counter + 3);
  noalloc_refresh_device(device);
  if (const char *tf = getenv("GBK_TUNE_FILE"))  // a tuned table saved by gbk_tune_save
    if (*tf) gbk_tune_load(c, tf);
  *out = c;
  return GBK_OK;
}

void gbk_destroy(gbk_ctx *c) {
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  c->release();
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  cudaGetLastError();
  delete c;
}

const char *gbk_last_error(const gbk_ctx *c) { return c ? c->err.c_str() : g_create_err.c_str(); }

int gbk_set_stream(gbk_ctx *c, void *stream) {
  if (!c) return GBK_ERR_ARG;
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return GBK_OK;
}

void *gbk_get_stream(const gbk_ctx *c) { return c ? (void *)c->stream : nullptr; }

int gbk_set_mode(gbk_ctx *c, int mode) {
  if (!c) return GBK_ERR_ARG;
  if (mode != GBK_MODE_F32C && mode != GBK_MODE_F64) return c->fail(GBK_ERR_ARG, "unknown mode %d", mode);
  c->mode = mode;
  return GBK_OK;
}

int gbk_get_mode(const gbk_ctx *c) { return c ? c->mode : -1; }

int gbk_set_order(gbk_ctx *c, int order) {
  if (!c) return GBK_ERR_ARG;
  if (order < GBK_ORDER_AUTO || order > GBK_ORDER_TWO_FLOAT)
    return c->fail(GBK_ERR_ARG, "unknown order %d", order);
  c->order = order;
  return GBK_OK;
}

int gbk_get_order(const gbk_ctx *c) { return c ? c->order : -1; }

int gbk_set_alloc_limit(gbk_ctx *c, size_t bytes) {
  if (!c) return GBK_ERR_ARG;
  c->alloc_limit = bytes;
  return GBK_OK;
}

int gbk_inject_pointer_device(gbk_ctx *c, int device) {
  if (!c || device < -1) return GBK_ERR_ARG;
  c->inject_pointer_device = device;
  return GBK_OK;
}

int gbk_set_gradient_mode(gbk_ctx *c, int mode) {
  if (!c) return GBK_ERR_ARG;
  if (mode != GBK_GRADIENT_REFERENCE && mode != GBK_GRADIENT_EXACT)
    return c->fail(GBK_ERR_ARG, "unknown gradient mode %d", mode);
  c->gradient_mode = mode;
  return GBK_OK;
}

int gbk_get_gradient_mode(const gbk_ctx *c) { return c ? c->gradient_mode : -1; }

int gbk_set_estimator(gbk_ctx *c, int estimator) {
  if (!c) return GBK_ERR_ARG;
  if (estimator != GBK_ESTIMATOR_FAST_GRADIENT_ASCENT && estimator != GBK_ESTIMATOR_GRADIENT_ASCENT)
    return c->fail(GBK_ERR_ARG, "unknown estimator %d", estimator);
  c->estimator = estimator;
  return GBK_OK;
}

int gbk_get_estimator(const gbk_ctx *c) { return c ? c->estimator : -1; }

int gbk_synchronize(gbk_ctx *c) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize")) return rc;
  unsigned st = 0;
  if (int rc = c->cuda(cudaMemcpy(&st, c->status, sizeof st, cudaMemcpyDeviceToHost), "status read")) return rc;
  if (st) {
    cudaMemset(c->status, 0, sizeof st);
    if (c->tickets.p) cudaMemset(c->tickets.p, 0, c->tickets.cap);  // a stopped CTA left its tile's count
    if (st & 2u)
      return c->fail(GBK_ERR_BOUNDS, "an index check of the bounds-checked build failed in a kernel sum since "
                     "the last check (the index was clamped); its outputs are not valid");
    return c->fail(GBK_ERR_TIMEOUT, "a bounded device-side wait gave up in a kernel sum since the last check; "
                   "its outputs are not valid");
  }
  return GBK_OK;
}

int gbk_set_staging(gbk_ctx *c, int staging) {
  if (!c) return GBK_ERR_ARG;
  if (staging < GBK_STAGING_AUTO || staging > GBK_STAGING_BULK) return c->fail(GBK_ERR_ARG, "unknown staging %d", staging);
  c->staging = staging;
  return GBK_OK;
}

int gbk_get_staging(const gbk_ctx *c) { return c ? c->staging : -1; }

int gbk_last_launch(const gbk_ctx *c, int *variant, int *nsplit) {
  if (!c) return GBK_ERR_ARG;
  if (variant) *variant = c->last_variant;
  if (nsplit) *nsplit = c->last_nsplit;
  return GBK_OK;
}

long long gbk_launch_count(const gbk_ctx *c) { return c ? c->launches : 0; }

int gbk_evaluated_pairs_by_op(gbk_ctx *c, long long *counts, int n) {
  if (!c || !c->pair_counter || !counts || n < 0) return GBK_ERR_ARG;
  if (cudaSetDevice(c->device) != cudaSuccess) {
    cudaGetLastError();
    return c->fail(GBK_ERR_CUDA, "cudaSetDevice(%d)", c->device);
  }
  unsigned long long v[OP_COUNT] = {0};
  if (int rc = c->cuda(cudaMemcpyAsync(v, c->pair_counter_of(0), sizeof v, cudaMemcpyDeviceToHost, c->stream),
                       "pair counters"))
    return rc;
  if (int rc = c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize")) return rc;
  for (int k = 0; k < n; ++k) counts[k] = k < OP_COUNT ? (long long)v[k] : 0;
  return GBK_OK;
}

long long gbk_evaluated_pairs(gbk_ctx *c) {
  long long v[OP_COUNT];
  if (gbk_evaluated_pairs_by_op(c, v, OP_COUNT) != GBK_OK) return -1;
  long long t = 0;
  for (long long x : v) t += x;
  return t;
}

// A device array the library owns for a caller that keeps no device memory of its own (the C++
// binding's per-object copies of the sources and weights).
struct gbk_buffer {
  int device = 0;
  double *p = nullptr;
  size_t cap = 0;  // doubles
  long long uploads = 0;
};

int gbk_buffer_create(gbk_ctx *c, gbk_buffer **out) {
  if (!c || !out) return GBK_ERR_ARG;
  *out = new gbk_buffer();
  (*out)->device = c->device;
  return GBK_OK;
}

int gbk_buffer_upload(gbk_ctx *c, gbk_buffer *b, const double *host, size_t count) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (!b || (count && !host)) return c->fail(GBK_ERR_ARG, "null pointer");
  if (b->device != c->device) return c->fail(GBK_ERR_ARG, "buffer of GPU %d, context on GPU %d", b->device, c->device);
  if (c->capturing()) return c->fail(GBK_ERR_STATE, "buffer upload while the stream is being captured");
  if (count > b->cap) {
    if (c->alloc_limit && count * sizeof(double) > c->alloc_limit)
      return c->fail(GBK_ERR_ALLOC, "buffer of %zu bytes refused (injected allocation limit)", count * sizeof(double));
    if (b->p) {
      if (int rc = c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize")) return rc;
      cudaFree(b->p);
      b->p = nullptr;
      b->cap = 0;
    }
    if (int rc = c->cuda(cudaMalloc(&b->p, count * sizeof(double)), "buffer allocation")) return rc;
    b->cap = count;
  }
  if (count) {
    if (int rc = c->cuda(cudaMemcpyAsync(b->p, host, count * sizeof(double), cudaMemcpyHostToDevice, c->stream),
                         "buffer upload"))
      return rc;
    if (int rc = c->cuda(cudaStreamSynchronize(c->stream), "cudaStreamSynchronize")) return rc;
  }
  ++b->uploads;
  return GBK_OK;
}

const double *gbk_buffer_data(const gbk_buffer *b) { return b ? b->p : nullptr; }

long long gbk_buffer_uploads(const gbk_buffer *b) { return b ? b->uploads : -1; }

void gbk_buffer_destroy(gbk_buffer *b) {
  if (!b) return;
  if (b->p) {
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(b->device);
    cudaDeviceSynchronize();
    cudaFree(b->p);
    cudaSetDevice(cur);
    cudaGetLastError();
  }
  delete b;
}

int gbk_set_split(gbk_ctx *c, int nsplit) {
  if (!c || nsplit < 0) return GBK_ERR_ARG;
  c->force_split = nsplit;
  return GBK_OK;
}

int gbk_convolve(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y,
                 const double *w, long ny, double sigma, double *out) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, dv, nx, ny, sigma)) return rc;
  if ((nx && (!x || !out)) || (ny && (!y || !w))) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  double *dout = io.out(out, (size_t)nx * dv, "out");
  if (io.rc) return io.rc;
  PairArgs a = base_args(nx, ny, sigma);
  a.x = dx;
  a.y = dy;
  if (int rc = run_chunked(c, OP_CONV, d, dv, a, dw, nullptr, dout, 1, nullptr)) return rc;
  return io.finish();
}

int gbk_convolve_gradient_alpha(gbk_ctx *c, int d, int dv, const double *x, long nx,
                                const double *y, const double *w, long ny, double sigma,
                                const double *alpha, double *out) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, dv, nx, ny, sigma)) return rc;
  if ((nx && (!x || !out || !alpha)) || (ny && (!y || !w))) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  const double *da = io.in(alpha, (size_t)nx * dv, "alpha");
  double *dout = io.out(out, (size_t)nx * d, "out");
  if (io.rc) return io.rc;
  PairArgs a = base_args(nx, ny, sigma);
  a.x = dx;
  a.y = dy;
  if (int rc = run_chunked(c, OP_GRADA, d, dv, a, dw, da, nullptr, 1, dout)) return rc;
  return io.finish();
}

int gbk_convolve_and_gradient_alpha(gbk_ctx *c, int d, int dv, const double *x, long nx,
                                    const double *y, const double *w, long ny, double sigma,
                                    const double *alpha, double *out_v, double *out_g) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, dv, nx, ny, sigma)) return rc;
  if ((nx && (!x || !out_v || !out_g || !alpha)) || (ny && (!y || !w)))
    return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  const double *da = io.in(alpha, (size_t)nx * dv, "alpha");
  double *dv_ = io.out(out_v, (size_t)nx * dv, "out_v");
  double *dg = io.out(out_g, (size_t)nx * d, "out_g");
  if (io.rc) return io.rc;
  PairArgs a = base_args(nx, ny, sigma);
  a.x = dx;
  a.y = dy;
  if (int rc = run_chunked(c, OP_CONV_GRADA, d, dv, a, dw, da, dv_, 1, dg)) return rc;
  return io.finish();
}

int gbk_convolve_gradient(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y,
                          const double *w, long ny, double sigma, double *out) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, dv, nx, ny, sigma)) return rc;
  if ((nx && (!x || !out)) || (ny && (!y || !w))) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  double *dout = io.out(out, (size_t)nx * dv * d, "out");
  if (io.rc) return io.rc;
  PairArgs a = base_args(nx, ny, sigma);
  a.x = dx;
  a.y = dy;
  if (int rc = run_chunked(c, OP_VARLIN, d, dv, a, dw, nullptr, dout, d, nullptr)) return rc;
  return io.finish();
}

int gbk_convolve_gradient_dim(gbk_ctx *c, int d, int dv, const double *x, long nx,
                              const double *y, const double *w, long ny, double sigma, int dim,
                              double *out) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, dv, nx, ny, sigma)) return rc;
  if (dim < 0 || dim >= d) return c->fail(GBK_ERR_ARG, "dimension index out of bounds");
  if ((nx && (!x || !out)) || (ny && (!y || !w))) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  double *dout = io.out(out, (size_t)nx * dv, "out");
  if (io.rc) return io.rc;
  PairArgs a = base_args(nx, ny, sigma);
  a.x = dx;
  a.y = dy;
  a.p0 = dim;
  if (int rc = run_chunked(c, OP_GRADDIM, d, dv, a, dw, nullptr, dout, 1, nullptr)) return rc;
  return io.finish();
}

int gbk_convolve_gradient_kdp(gbk_ctx *c, int d, int dv, const double *x, long nx,
                              const double *y, const double *w, long ny, double sigma, int k,
                              int dp, double *out) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, dv, nx, ny, sigma)) return rc;
  if (k < 0 || k >= dv) return c->fail(GBK_ERR_ARG, "Invalid weight index");
  if (dp < 0 || dp >= d) return c->fail(GBK_ERR_ARG, "Invalid derivative direction");
  if (nx < ny)
    return c->fail(GBK_ERR_ARG, "ConvolveGradient(X,k,dp) reads ny=%ld rows of X, which has %ld", ny, nx);
  if (ny && (!x || !y || !w || !out)) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)ny * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  double *dout = io.out(out, (size_t)ny, "out");
  if (io.rc) return io.rc;
  PairArgs a = base_args(ny, ny, sigma);  // the reference's target loop runs over ny rows
  a.x = dx;
  a.y = dy;
  a.p0 = dp;
  a.w = dw + k;
  a.w_ld = dv;
  a.out0 = dout;
  a.out0_ld = 1;
  if (int rc = c->launch(OP_GRADDIM, d, 1, a)) return rc;
  return io.finish();
}

int gbk_convolve_hessian(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y,
                         const double *w, long ny, double sigma, double *out) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, dv, nx, ny, sigma)) return rc;
  if ((nx && (!x || !out)) || (ny && (!y || !w))) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  double *dout = io.out(out, (size_t)nx * dv * d * d, "out");
  if (io.rc) return io.rc;
  PairArgs a = base_args(nx, ny, sigma);
  a.x = dx;
  a.y = dy;
  if (int rc = run_chunked(c, OP_HESSFULL, d, dv, a, dw, nullptr, dout, d * d, nullptr)) return rc;
  return io.finish();
}

int gbk_convolve_hessian_rowcol(gbk_ctx *c, int d, int dv, const double *x, long nx,
                                const double *y, const double *w, long ny, double sigma, int row,
                                int col, double *out) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, dv, nx, ny, sigma)) return rc;
  if (row < 0 || col < 0 || row >= d || col >= d) return c->fail(GBK_ERR_ARG, "Dimension index out of bounds");
  if ((nx && (!x || !out)) || (ny && (!y || !w))) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  double *dout = io.out(out, (size_t)nx * dv, "out");
  if (io.rc) return io.rc;
  PairArgs a = base_args(nx, ny, sigma);
  a.x = dx;
  a.y = dy;
  a.p0 = row;
  a.p1 = col;
  if (int rc = run_chunked(c, OP_HESSRC, d, dv, a, dw, nullptr, dout, 1, nullptr)) return rc;
  return io.finish();
}

int gbk_convolve_hessian_kdpdq(gbk_ctx *c, int d, int dv, const double *x, long nx,
                               const double *y, const double *w, long ny, double sigma, int k,
                               int dp, int dq, double *out) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, dv, nx, ny, sigma)) return rc;
  if (k < 0 || k >= dv) return c->fail(GBK_ERR_ARG, "Invalid weight index");
  if (dp < 0 || dq < 0 || dp >= d || dq >= d) return c->fail(GBK_ERR_ARG, "Invalid derivative direction");
  if ((nx && (!x || !out)) || (ny && (!y || !w))) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  double *dout = io.out(out, (size_t)nx, "out");
  if (io.rc) return io.rc;
  PairArgs a = base_args(nx, ny, sigma);
  a.x = dx;
  a.y = dy;
  a.p0 = dp;
  a.p1 = dq;
  a.w = dw + k;
  a.w_ld = dv;
  a.out0 = dout;
  a.out0_ld = 1;
  if (int rc = c->launch(OP_HESSRC, d, 1, a)) return rc;
  return io.finish();
}

int gbk_convolve_special_hessian(gbk_ctx *c, int d, const double *y, const double *w, long n,
                                 double sigma, const double *xi, double *out) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, d, n, n, sigma)) return rc;
  if (n && (!y || !w || !xi || !out)) return c->fail(GBK_ERR_ARG, "null pointer");
  HostIO io(c);
  const double *dy = io.in(y, (size_t)n * d, "y");
  const double *dw = io.in(w, (size_t)n * d, "w");
  const double *dxi = io.in(xi, (size_t)n * d, "xi");
  double *dout = io.out(out, (size_t)n * d, "out");
  if (io.rc) return io.rc;
  PairArgs a = base_args(n, n, sigma);
  a.x = dy;
  a.ta = dw;
  a.ta_ld = d;
  a.tb = dxi;
  a.tb_ld = d;
  a.y = dy;
  a.w = dw;
  a.w_ld = d;
  a.sb = dxi;
  a.sb_ld = d;
  a.out0 = dout;
  a.out0_ld = d;
  if (int rc = c->launch(OP_SPECIAL, d, d, a)) return rc;
  return io.finish();
}

int gbk_forward_adjoint(gbk_ctx *c, int d, int dv, const double *x, long nx, const double *y,
                        const double *w, long ny, double sigma, const double *alpha, double *v,
                        double *gx, double *gy, double *gw) {
  GBK_GUARD(c);
  GBK_RANGE();
  if (int rc = check_common(c, d, dv, nx, ny, sigma)) return rc;
  if ((nx && !x) || (ny && (!y || !w))) return c->fail(GBK_ERR_ARG, "null pointer");
  if ((gx || gy || gw) && nx && !alpha) return c->fail(GBK_ERR_ARG, "alpha is required for the adjoint");
  HostIO io(c);
  const double *dx = io.in(x, (size_t)nx * d, "x");
  const double *dy = io.in(y, (size_t)ny * d, "y");
  const double *dw = io.in(w, (size_t)ny * dv, "w");
  const double *da = io.in(alpha, (size_t)nx * dv, "alpha");
  double *dvv = io.out(v, (size_t)nx * dv, "v");
  double *dgx = io.out(gx, (size_t)nx * d, "gx");
  double *dgy = io.out(gy, (size_t)ny * d, "gy");
  double *dgw = io.out(gw, (size_t)ny * dv, "gw");
  if (io.rc) return io.rc;
  gbk_ctx::OrderCacheScope cache(c);  // both passes sort x and y: once each
  // target side: v = K w and gx (alpha-weighted gradient), one pass
  if (dvv || dgx) {
    PairArgs a = base_args(nx, ny, sigma);
    a.x = dx;
    a.y = dy;
    int op = (dvv && dgx) ? OP_CONV_GRADA : (dgx ? OP_GRADA : OP_CONV);
    if (int rc = run_chunked(c, op, d, dv, a, dw, op == OP_CONV ? nullptr : da, dvv, 1, dgx)) return rc;
  }
  // source side: roles swapped (targets y with "alpha" w, sources x with weights alpha)
  if (dgy || dgw) {
    PairArgs a = base_args(ny, nx, sigma);
    a.x = dy;
    a.y = dx;
    int op = (dgw && dgy) ? OP_CONV_GRADA : (dgy ? OP_GRADA : OP_CONV);
    if (int rc = run_chunked(c, op, d, dv, a, da, op == OP_CONV ? nullptr : dw, dgw, 1, dgy)) return rc;
  }
  return io.finish();
}

}  // extern "C"
