// Spatial order of point sets for the pair kernels: Morton keys, a stable radix sort, target tiles
// that never cross a coarse cell, and per-chunk bounding boxes of the sorted sources.
//
// Steps for n points (d = 2 or 3), all on the context's stream:
//  1. bounding box: per-block min/max, then one block over the block results;
//  2. keys: each coordinate quantised on a cubic grid over the box (10 bits a coordinate in 3-D,
//     15 in 2-D) and bit-interleaved into a 30-bit Morton key;
//  3. stable radix sort of (key, row) pairs (CUB), giving perm: sorted position -> row;
//  4a. targets: tiles of at most `tile` consecutive sorted points inside one cell of level L of
//      the Morton tree (2^L cells a side); a tile starts at every tile-th point of its cell. L is
//      the coarsest level whose cells are at most 16 units of the FP32 coordinate scale wide
//      (sqrt(log2 e) / sigma per input unit), at most 2^12 cells. So no CTA's bounding box is
//      wider than a cell, and the tiles number at most ceil(n / tile) + (non-empty cells): when
//      the whole set fits one such cell, the tiles are plain consecutive runs of the Morton order;
//  4b. sources: the bounding box of every `chunk` consecutive sorted sources, and a copy of the
//      source rows (coordinates, weights, extras) in sorted order, so the pair kernel stages
//      contiguous rows.
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

constexpr int kBoxBlocks = 256;  // blocks of the first bounding-box pass (at most)
constexpr int kThreads = 256;
constexpr int kKeyBits = 30;
constexpr double kCellWidth = 16.0;  // widest cell, in units of the FP32 coordinate scale

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

// Block-wide min/max of D pairs; the result is valid in thread 0.
template <int D>
__device__ void block_minmax(double *lo, double *hi) {
  __shared__ double s[2 * D][kThreads / 32];
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
    for (int w = 1; w < kThreads / 32; ++w)
#pragma unroll
      for (int l = 0; l < D; ++l) {
        lo[l] = fmin(lo[l], s[l][w]);
        hi[l] = fmax(hi[l], s[D + l][w]);
      }
}

template <int D>
__global__ void __launch_bounds__(kThreads) box_partial_kernel(const double *x, long n, double *part) {
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
  if (threadIdx.x == 0)
#pragma unroll
    for (int l = 0; l < D; ++l) {
      part[blockIdx.x * 2 * D + l] = lo[l];
      part[blockIdx.x * 2 * D + D + l] = hi[l];
    }
}

template <int D>
__global__ void __launch_bounds__(kThreads) box_final_kernel(const double *part, int nb, double *box) {
  double lo[D], hi[D];
#pragma unroll
  for (int l = 0; l < D; ++l) {
    lo[l] = 1e300;
    hi[l] = -1e300;
  }
  for (int b = threadIdx.x; b < nb; b += kThreads)
#pragma unroll
    for (int l = 0; l < D; ++l) {
      lo[l] = fmin(lo[l], part[b * 2 * D + l]);
      hi[l] = fmax(hi[l], part[b * 2 * D + D + l]);
    }
  block_minmax<D>(lo, hi);
  if (threadIdx.x == 0)
#pragma unroll
    for (int l = 0; l < D; ++l) {
      box[l] = lo[l];
      box[D + l] = hi[l];
    }
}

template <int D>
__global__ void __launch_bounds__(kThreads) keys_kernel(const double *x, long n, const double *box, unsigned *keys,
                                                        int *rows) {
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
  keys[i] = Morton<D>::key(q);
  rows[i] = (int)i;
}

// One thread per sorted position p: p opens a tile when it is a multiple of `tile` past the first
// position of its cell; the tile ends at the cell's end or `tile` positions later.
template <int D>
__global__ void __launch_bounds__(kThreads) tiles_kernel(const unsigned *keys, long n, const double *box,
                                                         double cell_scale, int tile, int2 *tiles, int *ntiles) {
  const long p = blockIdx.x * (long)kThreads + threadIdx.x;
  if (p >= n) return;
  double ext = 0.0;
#pragma unroll
  for (int l = 0; l < D; ++l) ext = fmax(ext, box[D + l] - box[l]);
  int level = 0;
  while (level < Morton<D>::kMaxLevel && ext * cell_scale > kCellWidth * (double)(1 << level)) ++level;
  const int shift = D * (Morton<D>::kBits - level);  // 0 < shift <= 30
  const unsigned cell = keys[p] >> shift;
  long lo = 0, hi = p;  // first position of the cell (keys ascending)
  while (lo < hi) {
    const long mid = (lo + hi) >> 1;
    if ((keys[mid] >> shift) < cell)
      lo = mid + 1;
    else
      hi = mid;
  }
  if ((p - lo) % tile != 0) return;
  long e_lo = p + 1, e_hi = p + tile < n ? p + tile : n;  // first position past the tile
  while (e_lo < e_hi) {
    const long mid = (e_lo + e_hi) >> 1;
    if ((keys[mid] >> shift) == cell)
      e_lo = mid + 1;
    else
      e_hi = mid;
  }
  const int k = atomicAdd(ntiles, 1);
  tiles[k] = make_int2((int)p, (int)e_lo);
}

// One warp per chunk of sorted sources: lo[D], hi[D] of the chunk.
template <int D>
__global__ void __launch_bounds__(kThreads) chunk_boxes_kernel(const double *y, const int *perm, long n, int chunk,
                                                               long nchunks, double *boxes) {
  const long c = (blockIdx.x * (long)kThreads + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (c >= nchunks) return;  // whole warp
  double lo[D], hi[D];
#pragma unroll
  for (int l = 0; l < D; ++l) {
    lo[l] = 1e300;
    hi[l] = -1e300;
  }
  const long end = (c + 1) * chunk < n ? (c + 1) * chunk : n;
  for (long q = c * chunk + lane; q < end; q += 32) {
    const long r = perm[q];
#pragma unroll
    for (int l = 0; l < D; ++l) {
      const double v = y[r * D + l];
      lo[l] = fmin(lo[l], v);
      hi[l] = fmax(hi[l], v);
    }
  }
#pragma unroll
  for (int l = 0; l < D; ++l)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo[l] = fmin(lo[l], __shfl_xor_sync(0xffffffffu, lo[l], o));
      hi[l] = fmax(hi[l], __shfl_xor_sync(0xffffffffu, hi[l], o));
    }
  if (lane == 0)
#pragma unroll
    for (int l = 0; l < D; ++l) {
      boxes[c * 2 * D + l] = lo[l];
      boxes[c * 2 * D + D + l] = hi[l];
    }
}

// dst[p, 0:cols] = src[perm[p] * ld + 0:cols] for p < n (dst row-major, `cols` wide).
__global__ void __launch_bounds__(kThreads) gather_rows_kernel(const double *src, int ld, int cols, const int *perm,
                                                               long n, double *dst) {
  const long t = blockIdx.x * (long)kThreads + threadIdx.x;
  if (t >= n * cols) return;
  const long p = t / cols;
  const int k = (int)(t - p * cols);
  dst[t] = src[(long)perm[p] * ld + k];
}

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

unsigned grid_for(long n) { return (unsigned)((n + kThreads - 1) / kThreads); }

// Morton sort of n points into perm (device, n ints). On return *keys_sorted and *box point into
// the context's order scratch, valid until the next order call on the stream.
template <int D>
int sort_points(gbk_ctx *c, const double *x, long n, int *perm, const unsigned **keys_sorted, const double **box) {
  if (n <= 0 || n >= INT_MAX) return c->fail(GBK_ERR_ARG, "spatial order: %ld points", n);
  const int nb = (int)std::min<long>(kBoxBlocks, (n + kThreads - 1) / kThreads);
  const size_t o_kout = al((size_t)n * 4), o_rows = o_kout + al((size_t)n * 4), o_part = o_rows + al((size_t)n * 4),
               o_box = o_part + al((size_t)kBoxBlocks * 2 * D * 8), total = o_box + al(2 * D * 8);
  if (int rc = c->ensure(c->order_tmp, total, "spatial order scratch")) return rc;
  char *base = (char *)c->order_tmp.p;
  unsigned *kin = (unsigned *)base, *kout = (unsigned *)(base + o_kout);
  int *rows = (int *)(base + o_rows);
  double *part = (double *)(base + o_part), *bx = (double *)(base + o_box);
  size_t cub_bytes = 0;
  if (int rc = c->cuda(cub::DeviceRadixSort::SortPairs(nullptr, cub_bytes, kin, kout, rows, perm, (int)n, 0,
                                                       kKeyBits, c->stream),
                       "radix sort size"))
    return rc;
  if (int rc = c->ensure(c->order_cub, std::max<size_t>(cub_bytes, 256), "radix sort scratch")) return rc;
  box_partial_kernel<D><<<nb, kThreads, 0, c->stream>>>(x, n, part);
  box_final_kernel<D><<<1, kThreads, 0, c->stream>>>(part, nb, bx);
  keys_kernel<D><<<grid_for(n), kThreads, 0, c->stream>>>(x, n, bx, kin, rows);
  if (int rc = c->cuda(cudaGetLastError(), "spatial order keys")) return rc;
  size_t bytes = c->order_cub.cap;
  if (int rc = c->cuda(cub::DeviceRadixSort::SortPairs(c->order_cub.p, bytes, kin, kout, rows, perm, (int)n, 0,
                                                       kKeyBits, c->stream),
                       "radix sort"))
    return rc;
  *keys_sorted = kout;
  *box = bx;
  return GBK_OK;
}

template <int D>
int targets_impl(gbk_ctx *c, const double *x, long n, int tile, double sigma, OrderView *out) {
  const long bound = (n + tile - 1) / tile + std::min<long>(n, 1L << (D * Morton<D>::kMaxLevel));
  const size_t o_tiles = al((size_t)n * 4), o_cnt = o_tiles + al((size_t)bound * 8), total = o_cnt + 256;
  if (int rc = c->ensure(c->order_keep[0], total, "target order")) return rc;
  char *base = (char *)c->order_keep[0].p;
  int *perm = (int *)base;
  int2 *tiles = (int2 *)(base + o_tiles);
  int *cnt = (int *)(base + o_cnt);
  const unsigned *keys;
  const double *box;
  if (int rc = sort_points<D>(c, x, n, perm, &keys, &box)) return rc;
  if (int rc = c->cuda(cudaMemsetAsync(cnt, 0, sizeof(int), c->stream), "tile count reset")) return rc;
  tiles_kernel<D><<<grid_for(n), kThreads, 0, c->stream>>>(keys, n, box, coord_scale<float>(sigma), tile, tiles,
                                                           cnt);
  if (int rc = c->cuda(cudaGetLastError(), "target tiles")) return rc;
  out->perm = perm;
  out->tiles = tiles;
  out->ntiles = cnt;
  out->tile_bound = bound;
  out->boxes = nullptr;
  return GBK_OK;
}

template <int D>
int sources_impl(gbk_ctx *c, const double *y, long n, int chunk, OrderView *out) {
  const long nchunks = (n + chunk - 1) / chunk;
  const size_t o_box = al((size_t)n * 4), total = o_box + al((size_t)nchunks * 2 * D * 8);
  if (int rc = c->ensure(c->order_keep[1], total, "source order")) return rc;
  char *base = (char *)c->order_keep[1].p;
  int *perm = (int *)base;
  double *boxes = (double *)(base + o_box);
  const unsigned *keys;
  const double *box;
  if (int rc = sort_points<D>(c, y, n, perm, &keys, &box)) return rc;
  chunk_boxes_kernel<D><<<grid_for(nchunks * 32), kThreads, 0, c->stream>>>(y, perm, n, chunk, nchunks, boxes);
  if (int rc = c->cuda(cudaGetLastError(), "source chunk boxes")) return rc;
  out->perm = perm;
  out->tiles = nullptr;
  out->ntiles = nullptr;
  out->tile_bound = 0;
  out->boxes = boxes;
  return GBK_OK;
}

}  // namespace

int gather_sources(gbk_ctx *c, const int *perm, long n, const double *const *src, const int *ld, const int *cols,
                   int narrays, double **dst) {
  size_t total = 0;
  for (int k = 0; k < narrays; ++k) total += al((size_t)n * cols[k] * sizeof(double));
  if (int rc = c->ensure(c->order_src, total, "sorted source copy")) return rc;
  char *base = (char *)c->order_src.p;
  for (int k = 0; k < narrays; ++k) {
    dst[k] = (double *)base;
    base += al((size_t)n * cols[k] * sizeof(double));
    gather_rows_kernel<<<grid_for(n * cols[k]), kThreads, 0, c->stream>>>(src[k], ld[k], cols[k], perm, n, dst[k]);
  }
  return c->cuda(cudaGetLastError(), "sorted source copy");
}

int order_targets(gbk_ctx *c, int d, const double *x, long n, int tile, double sigma, OrderView *out) {
  if (tile <= 0) return c->fail(GBK_ERR_ARG, "spatial order: tile %d", tile);
  return d == 3 ? targets_impl<3>(c, x, n, tile, sigma, out) : targets_impl<2>(c, x, n, tile, sigma, out);
}

int order_sources(gbk_ctx *c, int d, const double *y, long n, int chunk, OrderView *out) {
  if (chunk <= 0) return c->fail(GBK_ERR_ARG, "spatial order: chunk %d", chunk);
  return d == 3 ? sources_impl<3>(c, y, n, chunk, out) : sources_impl<2>(c, y, n, chunk, out);
}

}  // namespace gbk
