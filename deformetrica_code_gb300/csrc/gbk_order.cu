// Spatial order of point sets for the pair kernels: Morton keys, a stable radix sort, target tiles
// that never cross a coarse cell, per-chunk bounding boxes and sorted copies of the sources.
//
// Steps for n points (d = 2 or 3), all on the context's stream:
//  1. bounding box: per-block min/max; the last block to finish reduces the block results
//     (one launch, a self-resetting ticket in device memory);
//  2. keys: each coordinate quantised on a cubic grid over the box (10 bits a coordinate in 3-D,
//     15 in 2-D) and bit-interleaved into a 30-bit Morton key;
//  3. sort of (key, row) pairs, giving perm: sorted position -> row. Up to kSmallMax points: the
//     level-kMaxLevel cell (the key's top 12 bits) sorted by one CTA (block radix sort); above:
//     CUB's device radix sort of the full key. Inside one API call that opts in, a point set sorted
//     once is reused (the forward + adjoint passes sort x and y once each);
//  4a. targets: tiles of at most `tile` consecutive sorted points inside one cell of level L of
//      the Morton tree (2^L cells a side); a tile starts at every tile-th point of its cell. L is
//      the coarsest level whose cells are at most 16 units of the FP32 coordinate scale wide
//      (sqrt(log2 e) / sigma per input unit), at most 2^12 cells. So no CTA's bounding box is
//      wider than a cell, and the tiles number at most ceil(n / tile) + (non-empty cells): when
//      the whole set fits one such cell, the tiles are plain runs of the sorted order;
//  4b. sources: the bounding box of every `chunk` consecutive sorted sources, written with sorted
//      copies of the source rows the pair kernel stages (coordinates, weights, extras), one CTA
//      per chunk and one thread per row.
// GB300 runs FP64 at a small fraction of its FP32 rate, so every FP64 step (boxes, quantisation)
// is spread over many CTAs; the single-CTA sort works on integer keys only.
#include <cuda_runtime.h>

#include <cub/cub.cuh>

#include <algorithm>
#include <climits>

#include "../../include/gbk.h"
#include "gbk_common.cuh"
#include "gbk_ctx.h"
#include "gbk_order.h"

namespace gbk {
namespace {

constexpr int kBoxBlocks = 256;  // blocks of the bounding-box kernel (at most)
constexpr int kThreads = 256;
constexpr int kKeyBits = 30;
constexpr double kCellWidth = 16.0;  // widest cell, in units of the FP32 coordinate scale
constexpr int kCellBits = 12;        // cell keys of the single-CTA sort: kMaxLevel levels

template <int D>
struct Morton;
template <>
struct Morton<3> {
  static constexpr int kBits = 10;
  static constexpr int kMaxLevel = 4;  // 4096 cells
  __device__ static unsigned spread(unsigned v) {  // bit k -> bit 3k
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000ffu;
    v = (v | (v << 8)) & 0x0300f00fu;
    v = (v | (v << 4)) & 0x030c30c3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
  }
  __device__ static unsigned key(const unsigned *q) {
    return (spread(q[0]) << 2) | (spread(q[1]) << 1) | spread(q[2]);
  }
};
template <>
struct Morton<2> {
  static constexpr int kBits = 15;
  static constexpr int kMaxLevel = 6;  // 4096 cells
  __device__ static unsigned spread(unsigned v) {  // bit k -> bit 2k
    v &= 0x7fffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
  }
  __device__ static unsigned key(const unsigned *q) { return (spread(q[0]) << 1) | spread(q[1]); }
};

// Block-wide min/max of D pairs over NT threads; the result is valid in thread 0.
template <int D, int NT = kThreads>
__device__ void block_minmax(double *lo, double *hi) {
  __shared__ double s[2 * D][NT / 32];
#pragma unroll
  for (int l = 0; l < D; ++l)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[l] = fmin(lo[l], __shfl_xor_sync(0xffffffffu, lo[l], o));
      hi[l] = fmax(hi[l], __shfl_xor_sync(0xffffffffu, hi[l], o));
    }
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int l = 0; l < D; ++l) {
      s[l][threadIdx.x >> 5] = lo[l];
      s[D + l][threadIdx.x >> 5] = hi[l];
    }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int w = 1; w < NT / 32; ++w)
#pragma unroll
      for (int l = 0; l < D; ++l) {
        lo[l] = fmin(lo[l], s[l][w]);
        hi[l] = fmax(hi[l], s[D + l][w]);
      }
}

// Bounding box: block results in part[], the last block reduces them into box[] and resets the
// ticket for the next call.
template <int D>
__global__ void __launch_bounds__(kThreads) box_kernel(const double *x, long n, double *part, double *box,
                                                       unsigned *ticket) {
  pdl_entry();
  __shared__ bool last;
  double lo[D], hi[D];
#pragma unroll
  for (int l = 0; l < D; ++l) {
    lo[l] = 1e300;
    hi[l] = -1e300;
  }
  for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < n; i += (long)gridDim.x * kThreads)
#pragma unroll
    for (int l = 0; l < D; ++l) {
      const double v = x[i * D + l];
      lo[l] = fmin(lo[l], v);
      hi[l] = fmax(hi[l], v);
    }
  block_minmax<D>(lo, hi);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int l = 0; l < D; ++l) {
      part[blockIdx.x * 2 * D + l] = lo[l];
      part[blockIdx.x * 2 * D + D + l] = hi[l];
    }
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
#pragma unroll
  for (int l = 0; l < D; ++l) {
    lo[l] = 1e300;
    hi[l] = -1e300;
  }
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads)
#pragma unroll
    for (int l = 0; l < D; ++l) {
      lo[l] = fmin(lo[l], __ldcg(part + b * 2 * D + l));
      hi[l] = fmax(hi[l], __ldcg(part + b * 2 * D + D + l));
    }
  block_minmax<D>(lo, hi);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int l = 0; l < D; ++l) {
      box[l] = lo[l];
      box[D + l] = hi[l];
    }
    *ticket = 0u;
  }
}

// Bounding box of the union of two point sets (x then y, one grid-stride loop over both), with the
// same last-block reduction and self-resetting ticket as box_kernel.
template <int D>
__global__ void __launch_bounds__(kThreads) union_box_kernel(const double *x, long nx, const double *y, long ny,
                                                             double *part, double *box, unsigned *ticket) {
  pdl_entry();
  __shared__ bool last;
  double lo[D], hi[D];
#pragma unroll
  for (int l = 0; l < D; ++l) {
    lo[l] = 1e300;
    hi[l] = -1e300;
  }
  const long n = nx + ny;
  for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < n; i += (long)gridDim.x * kThreads) {
    const double *p = i < nx ? x + i * D : y + (i - nx) * D;
#pragma unroll
    for (int l = 0; l < D; ++l) {
      lo[l] = fmin(lo[l], p[l]);
      hi[l] = fmax(hi[l], p[l]);
    }
  }
  block_minmax<D>(lo, hi);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int l = 0; l < D; ++l) {
      part[blockIdx.x * 2 * D + l] = lo[l];
      part[blockIdx.x * 2 * D + D + l] = hi[l];
    }
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
#pragma unroll
  for (int l = 0; l < D; ++l) {
    lo[l] = 1e300;
    hi[l] = -1e300;
  }
  for (int b = threadIdx.x; b < (int)gridDim.x; b += kThreads)
#pragma unroll
    for (int l = 0; l < D; ++l) {
      lo[l] = fmin(lo[l], __ldcg(part + b * 2 * D + l));
      hi[l] = fmax(hi[l], __ldcg(part + b * 2 * D + D + l));
    }
  block_minmax<D>(lo, hi);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int l = 0; l < D; ++l) {
      box[l] = lo[l];
      box[D + l] = hi[l];
    }
    *ticket = 0u;
  }
}

// Morton key of every point, shifted right by `shift` bits (0: full key; 18: level-kMaxLevel cell).
template <int D>
__global__ void __launch_bounds__(kThreads) keys_kernel(const double *x, long n, const double *box, int shift,
                                                        unsigned *keys, int *rows) {
  pdl_entry();
  const long i = blockIdx.x * (long)kThreads + threadIdx.x;
  if (i >= n) return;
  double ext = 0.0;
#pragma unroll
  for (int l = 0; l < D; ++l) ext = fmax(ext, box[D + l] - box[l]);
  constexpr unsigned kCells = 1u << Morton<D>::kBits;
  const double scale = ext > 0.0 ? (double)kCells / ext : 0.0;
  unsigned q[D];
#pragma unroll
  for (int l = 0; l < D; ++l) {
    const double t = fmin(fmax((x[i * D + l] - box[l]) * scale, 0.0), (double)(kCells - 1));
    q[l] = (unsigned)t;
  }
  keys[i] = Morton<D>::key(q) >> shift;
  if (rows) rows[i] = (int)i;
}

// Level of the target cells: the coarsest whose width is at most kCellWidth scaled units.
template <int D>
__device__ int cell_level(const double *box, double cell_scale) {
  double ext = 0.0;
#pragma unroll
  for (int l = 0; l < D; ++l) ext = fmax(ext, box[D + l] - box[l]);
  int level = 0;
  while (level < Morton<D>::kMaxLevel && ext * cell_scale > kCellWidth * (double)(1 << level)) ++level;
  return level;
}

// Tile of sorted position p (keys ascending, cell = key >> shift): whether p opens a tile, and the
// first position past it.
__device__ bool tile_at(const unsigned *keys, long n, long p, int shift, int tile, long *end) {
  const unsigned cell = keys[p] >> shift;
  long lo = 0, hi = p;  // first position of the cell
  while (lo < hi) {
    const long mid = (lo + hi) >> 1;
    if ((keys[mid] >> shift) < cell)
      lo = mid + 1;
    else
      hi = mid;
  }
  if ((p - lo) % tile != 0) return false;
  long e_lo = p + 1, e_hi = p + tile < n ? p + tile : n;
  while (e_lo < e_hi) {
    const long mid = (e_lo + e_hi) >> 1;
    if ((keys[mid] >> shift) == cell)
      e_lo = mid + 1;
    else
      e_hi = mid;
  }
  *end = e_lo;
  return true;
}

// Target tiles over sorted keys of `key_bits` bits (30: full Morton keys; 12: level-kMaxLevel
// cells), one thread per sorted position; tiles are appended in any order.
template <int D>
__global__ void __launch_bounds__(kThreads) tiles_kernel(const unsigned *keys, long n, int key_bits, const double *box,
                                                         double cell_scale, int tile, int2 *tiles, int *ntiles) {
  pdl_entry();
  const long p = blockIdx.x * (long)kThreads + threadIdx.x;
  if (p >= n) return;
  const int shift = key_bits - D * cell_level<D>(box, cell_scale);  // 0 < shift <= key_bits
  long end;
  if (!tile_at(keys, n, p, shift, tile, &end)) return;
  tiles[atomicAdd(ntiles, 1)] = make_int2((int)p, (int)end);
}

// ---- single-CTA sort of cell keys (n <= kSmallThreads * ITEMS) ----
constexpr int kSmallThreads = 1024;
constexpr int kSmallMax = kSmallThreads * 16;

template <int ITEMS>
struct SmallSort {
  typedef cub::BlockRadixSort<unsigned, kSmallThreads, ITEMS, int> Sort;
};

// Sorts the n cell keys with their rows: sorted keys and perm. Keys of points t + k * kSmallThreads
// go to thread t's k-th item, so ties keep that fixed order.
template <int ITEMS>
__global__ void __launch_bounds__(kSmallThreads, 1)
    small_sort_kernel(const unsigned *cell_keys, int n, unsigned *sorted_keys, int *perm) {
  pdl_entry();
  typedef typename SmallSort<ITEMS>::Sort Sort;
  extern __shared__ __align__(16) unsigned char small_smem[];
  const int t = threadIdx.x;
  unsigned keys[ITEMS];
  int rows[ITEMS];
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int i = t + k * kSmallThreads;
    rows[k] = i;
    keys[k] = i < n ? cell_keys[i] : (1u << kCellBits);  // padding sorts last
  }
  Sort(*reinterpret_cast<typename Sort::TempStorage *>(small_smem)).Sort(keys, rows, 0, kCellBits + 1);
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const int p = t * ITEMS + k;
    if (p < n) {
      sorted_keys[p] = keys[k];
      perm[p] = rows[k];
    }
  }
}

// One CTA per chunk of sorted sources, one thread per row: the chunk's box and the sorted copies.
template <int D>
__global__ void source_pack_kernel(const double *y, const int *perm, long n, int chunk, double *boxes,
                                   SourceCopies sc) {
  pdl_entry();
  __shared__ double s[2 * D][kThreads / 32];
  const long c = blockIdx.x;
  double lo[D], hi[D];
#pragma unroll
  for (int l = 0; l < D; ++l) {
    lo[l] = 1e300;
    hi[l] = -1e300;
  }
  const long end = (c + 1) * chunk < n ? (c + 1) * chunk : n;
  bool bad = false;  // a non-finite coordinate or source value in the chunk
  for (long q = c * chunk + threadIdx.x; q < end; q += blockDim.x) {
    const long r = perm[q];
#pragma unroll
    for (int l = 0; l < D; ++l) {
      const double v = y[r * D + l];
      lo[l] = fmin(lo[l], v);
      hi[l] = fmax(hi[l], v);
      bad = bad || !isfinite(v);
      if (sc.dst[0]) sc.dst[0][q * D + l] = v;
    }
    for (int k = 1; k < sc.na; ++k)
      for (int j = 0; j < sc.cols[k]; ++j) {
        const double v = sc.src[k][r * sc.ld[k] + j];
        bad = bad || !isfinite(v);
        sc.dst[k][q * sc.cols[k] + j] = v;
      }
    for (int k = 0; k < 3; ++k)
      if (sc.chk[k])
        for (int j = 0; j < sc.chk_cols[k]; ++j) bad = bad || !isfinite(sc.chk[k][r * sc.chk_ld[k] + j]);
  }
  const bool chunk_bad = __syncthreads_or(bad) != 0;
#pragma unroll
  for (int l = 0; l < D; ++l)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[l] = fmin(lo[l], __shfl_xor_sync(0xffffffffu, lo[l], o));
      hi[l] = fmax(hi[l], __shfl_xor_sync(0xffffffffu, hi[l], o));
    }
  const int warps = (blockDim.x + 31) >> 5;
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int l = 0; l < D; ++l) {
      s[l][threadIdx.x >> 5] = lo[l];
      s[D + l][threadIdx.x >> 5] = hi[l];
    }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < warps; ++w)
#pragma unroll
      for (int l = 0; l < D; ++l) {
        lo[l] = fmin(lo[l], s[l][w]);
        hi[l] = fmax(hi[l], s[D + l][w]);
      }
#pragma unroll
    for (int l = 0; l < D; ++l) {  // an unbounded box for a chunk that must be visited
      boxes[c * 2 * D + l] = chunk_bad ? -INFINITY : lo[l];
      boxes[c * 2 * D + D + l] = chunk_bad ? INFINITY : hi[l];
    }
  }
}

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

unsigned grid_for(long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

template <int ITEMS>
cudaError_t launch_small_sort(cudaStream_t st, const unsigned *keys, long n, unsigned *sorted, int *perm) {
  auto kern = small_sort_kernel<ITEMS>;
  constexpr size_t smem = sizeof(typename SmallSort<ITEMS>::Sort::TempStorage);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  kern<<<1, kSmallThreads, smem, st>>>(keys, (int)n, sorted, perm);
  return cudaGetLastError();
}

// Steps 1-3 for n points into slot `s`: perm, sorted keys and box.
template <int D>
int sort_into(gbk_ctx *c, gbk_ctx::SortSlot &s, const double *x, long n, SortedSet *out) {
  if (n <= 0 || n >= INT_MAX) return c->fail(GBK_ERR_ARG, "spatial order: %ld points", n);
  const bool small = n <= kSmallMax;
  const int nb = (int)std::min<long>(kBoxBlocks, (n + kThreads - 1) / kThreads);
  // slot: perm | sorted keys | box;  scratch: keys | rows | block boxes
  const size_t o_keys = al((size_t)n * 4), o_box = o_keys + al((size_t)n * 4), slot_bytes = o_box + al(2 * D * 8);
  const size_t o_rows = al((size_t)n * 4), o_part = o_rows + al((size_t)n * 4),
               tmp_bytes = o_part + al((size_t)kBoxBlocks * 2 * D * 8);
  if (int rc = c->ensure(s.buf, slot_bytes, "spatial order")) return rc;
  if (int rc = c->ensure(c->order_tmp, tmp_bytes, "spatial order scratch")) return rc;
  char *sb = (char *)s.buf.p, *tb = (char *)c->order_tmp.p;
  int *perm = (int *)sb;
  unsigned *sorted = (unsigned *)(sb + o_keys);
  double *box = (double *)(sb + o_box);
  unsigned *kin = (unsigned *)tb;
  int *rows = (int *)(tb + o_rows);
  double *part = (double *)(tb + o_part);
  if (!small) {
    size_t cub_bytes = 0;
    if (int rc = c->cuda(cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, kin, sorted, rows, perm, (int)n, 0,
                                                         kKeyBits, c->stream),
                         "radix sort size"))
      return rc;
    if (int rc = c->ensure(c->order_cub, std::max<size_t>(cub_bytes, 256), "radix sort scratch")) return rc;
  }
  box_kernel<D><<<nb, kThreads, 0, c->stream>>>(x, n, part, box, c->order_ticket);
  keys_kernel<D><<<grid_for(n), kThreads, 0, c->stream>>>(x, n, box, small ? kKeyBits - kCellBits : 0, kin,
                                                          small ? nullptr : rows);
  if (int rc = c->cuda(cudaGetLastError(), "spatial order keys")) return rc;
  out->launches = 2;
  if (small) {
    cudaError_t e = n <= kSmallThreads * 4   ? launch_small_sort<4>(c->stream, kin, n, sorted, perm)
                    : n <= kSmallThreads * 8 ? launch_small_sort<8>(c->stream, kin, n, sorted, perm)
                                             : launch_small_sort<16>(c->stream, kin, n, sorted, perm);
    if (int rc = c->cuda(e, "spatial order sort")) return rc;
    out->launches = 3;
  } else {
    size_t bytes = c->order_cub.cap;
    if (int rc = c->cuda(cub::DeviceRadixSort::SortPairs(c->order_cub.p, bytes, kin, sorted, rows, perm, (int)n, 0,
                                                         kKeyBits, c->stream),
                         "radix sort"))
      return rc;
  }
  s.ptr = x;
  s.n = n;
  s.d = D;
  s.epoch = c->call_epoch;
  s.key_bits = small ? kCellBits : kKeyBits;
  out->perm = perm;
  out->keys = sorted;
  out->box = box;
  out->n = n;
  out->key_bits = s.key_bits;
  return GBK_OK;
}

}  // namespace

__global__ void __launch_bounds__(kThreads) nonfinite_kernel(int d, const double *x, long n, const double *a, int lda,
                                                             const double *b, int ldb, const double *e, int lde,
                                                             unsigned *flag) {
  pdl_entry();
  bool bad = false;
  for (long i = blockIdx.x * (long)kThreads + threadIdx.x; i < n; i += (long)gridDim.x * kThreads) {
    for (int k = 0; k < d; ++k) bad = bad || !isfinite(x[i * d + k]);
    if (a)
      for (int k = 0; k < lda; ++k) bad = bad || !isfinite(a[i * lda + k]);
    if (b)
      for (int k = 0; k < ldb; ++k) bad = bad || !isfinite(b[i * ldb + k]);
    if (e)
      for (int k = 0; k < lde; ++k) bad = bad || !isfinite(e[i * lde + k]);
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flag, 1u);
}

// boxes: lo[d], hi[d] per chunk -> (-inf, +inf) when *flag
__global__ void unbound_boxes_kernel(const unsigned *flag, double *boxes, long nvals, int d) {
  pdl_entry();
  if (!*flag) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < nvals; i += (long)gridDim.x * blockDim.x)
    boxes[i] = (i % (2 * d)) < d ? -INFINITY : INFINITY;
}

cudaError_t unbound_boxes_if_nonfinite(cudaStream_t st, int d, const double *x, long n, const double *a, int lda,
                                       const double *b, int ldb, const double *e, int lde, unsigned *flag,
                                       double *boxes, long nchunks) {
  cudaError_t err = cudaMemsetAsync(flag, 0, sizeof(unsigned), st);
  if (err != cudaSuccess) return err;
  const long blocks = std::min<long>(std::max<long>((n + kThreads - 1) / kThreads, 1), 1216);
  nonfinite_kernel<<<(unsigned)blocks, kThreads, 0, st>>>(d, x, n, a, lda, b, ldb, e, lde, flag);
  if ((err = cudaGetLastError()) != cudaSuccess) return err;
  const long nvals = nchunks * 2 * d;
  const long bb = std::min<long>(std::max<long>((nvals + kThreads - 1) / kThreads, 1), 1216);
  unbound_boxes_kernel<<<(unsigned)bb, kThreads, 0, st>>>(flag, boxes, nvals, d);
  return cudaGetLastError();
}

int order_extent(gbk_ctx *c, int d, const double *x, long nx, const double *y, long ny, double *extent) {
  *extent = 0.0;
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "spatial order: dimension %d", d);
  if (!c->host_box) return c->fail(GBK_ERR_STATE, "spatial order: no pinned read-back buffer");
  const size_t o_box = al((size_t)kBoxBlocks * 2 * 3 * 8);
  if (int rc = c->ensure(c->order_box, o_box + al(2 * 3 * 8), "extent scratch")) return rc;
  double *part = (double *)c->order_box.p;
  double *box = (double *)((char *)c->order_box.p + o_box);
  const long n = nx + ny;
  const int nb = (int)std::max<long>(1, std::min<long>(kBoxBlocks, (n + kThreads - 1) / kThreads));
  if (d == 3)
    union_box_kernel<3><<<nb, kThreads, 0, c->stream>>>(x, nx, y, ny, part, box, c->order_ticket);
  else
    union_box_kernel<2><<<nb, kThreads, 0, c->stream>>>(x, nx, y, ny, part, box, c->order_ticket);
  if (int rc = c->cuda(cudaGetLastError(), "extent box")) return rc;
  c->launches += 1;
  if (int rc = c->cuda(cudaMemcpyAsync(c->host_box, box, 2 * d * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
                       "extent read-back"))
    return rc;
  if (int rc = c->cuda(cudaStreamSynchronize(c->stream), "extent read-back")) return rc;
  double e = 0.0;
  for (int l = 0; l < d; ++l) {
    const double lo = c->host_box[l], hi = c->host_box[d + l];
    if (lo <= hi) e = std::max(e, hi - lo);  // NaN coordinates are ignored by the box, as by the sort
  }
  *extent = e;
  return GBK_OK;
}

int order_sort(gbk_ctx *c, int d, const double *x, long n, SortedSet *out) {
  *out = SortedSet();
  if (d != 2 && d != 3) return c->fail(GBK_ERR_UNSUPPORTED, "spatial order: dimension %d", d);
  // a sort of the same rows earlier in this call (inside an order-cache scope)
  if (c->order_cache)
    for (auto &s : c->sort_slot)
      if (s.ptr == x && s.n == n && s.d == d && s.epoch == c->call_epoch) {
        const size_t o_keys = al((size_t)n * 4), o_box = o_keys + al((size_t)n * 4);
        char *sb = (char *)s.buf.p;
        out->perm = (const int *)sb;
        out->keys = (const unsigned *)(sb + o_keys);
        out->box = (const double *)(sb + o_box);
        out->n = n;
        out->key_bits = s.key_bits;
        s.last_use = ++c->sort_clock;
        return GBK_OK;
      }
  // otherwise the least recently used slot
  gbk_ctx::SortSlot *slot = &c->sort_slot[0];
  for (auto &s : c->sort_slot)
    if (s.last_use < slot->last_use) slot = &s;
  slot->last_use = ++c->sort_clock;
  slot->ptr = nullptr;
  return d == 3 ? sort_into<3>(c, *slot, x, n, out) : sort_into<2>(c, *slot, x, n, out);
}

int order_targets(gbk_ctx *c, int d, const SortedSet &s, int tile, double sigma, OrderView *out) {
  if (tile <= 0) return c->fail(GBK_ERR_ARG, "spatial order: tile %d", tile);
  const long n = s.n;
  const int max_level = d == 3 ? Morton<3>::kMaxLevel : Morton<2>::kMaxLevel;
  const long bound = (n + tile - 1) / tile + std::min<long>(n, 1L << (d * max_level));
  const size_t o_cnt = al((size_t)bound * 8), total = o_cnt + 256;
  if (int rc = c->ensure(c->order_keep[0], total, "target tiles")) return rc;
  char *base = (char *)c->order_keep[0].p;
  int2 *tiles = (int2 *)base;
  int *cnt = (int *)(base + o_cnt);
  *out = OrderView();
  out->perm = s.perm;
  out->tiles = tiles;
  out->ntiles = cnt;
  out->tile_bound = bound;
  // the usual count is ceil(n / tile) plus a partial tile per non-empty cell; more loop
  const long full = (n + tile - 1) / tile;
  out->grid = std::min(bound, 3 * full + 2L * c->num_sms);
  out->launches = 1;
  if (int rc = c->cuda(cudaMemsetAsync(cnt, 0, sizeof(int), c->stream), "tile count reset")) return rc;
  const double cs = coord_scale<float>(sigma);
  if (d == 3)
    tiles_kernel<3><<<grid_for(n), kThreads, 0, c->stream>>>(s.keys, n, s.key_bits, s.box, cs, tile, tiles, cnt);
  else
    tiles_kernel<2><<<grid_for(n), kThreads, 0, c->stream>>>(s.keys, n, s.key_bits, s.box, cs, tile, tiles, cnt);
  return c->cuda(cudaGetLastError(), "target tiles");
}

int order_sources(gbk_ctx *c, int d, const double *y, const SortedSet &s, int chunk, const SourceCopies &want,
                  OrderView *out) {
  if (chunk <= 0 || chunk % 32 != 0) return c->fail(GBK_ERR_ARG, "spatial order: chunk %d", chunk);
  if (want.na < 0 || want.na > 3) return c->fail(GBK_ERR_ARG, "spatial order: %d source copies", want.na);
  const long n = s.n, nchunks = (n + chunk - 1) / chunk;
  if (int rc = c->ensure(c->order_keep[1], al((size_t)nchunks * 2 * d * 8), "source boxes")) return rc;
  SourceCopies sc = want;
  // every copy is padded to whole chunks, so a chunk can be fetched whole (bulk staging); the rows
  // past n are never used
  const size_t npad = (size_t)nchunks * chunk;
  size_t copy_bytes = 0;
  for (int k = 0; k < sc.na; ++k) copy_bytes += al(npad * sc.cols[k] * sizeof(double));
  if (copy_bytes)
    if (int rc = c->ensure(c->order_src, copy_bytes, "sorted source copies")) return rc;
  char *cb = (char *)c->order_src.p;
  for (int k = 0; k < 3; ++k) {
    sc.dst[k] = nullptr;
    if (k < sc.na) {
      sc.dst[k] = (double *)cb;
      cb += al(npad * sc.cols[k] * sizeof(double));
    }
  }
  double *boxes = (double *)c->order_keep[1].p;
  *out = OrderView();
  out->perm = s.perm;
  out->boxes = boxes;
  for (int k = 0; k < 3; ++k) out->copies[k] = sc.dst[k];
  out->launches = 1;
  const int threads = std::min(chunk, kThreads);
  if (d == 3)
    source_pack_kernel<3><<<(unsigned)nchunks, threads, 0, c->stream>>>(y, s.perm, n, chunk, boxes, sc);
  else
    source_pack_kernel<2><<<(unsigned)nchunks, threads, 0, c->stream>>>(y, s.perm, n, chunk, boxes, sc);
  return c->cuda(cudaGetLastError(), "source boxes and copies");
}

}  // namespace gbk
