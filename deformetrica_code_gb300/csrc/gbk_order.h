// Spatial order of a point set for the pair kernels (gbk_order.cu).
//
// The FP32 lanes centre coordinates on each CTA's target bounding box, so the rounding error of a
// pair's x - y grows with the distance of the target from that centre. With targets in caller
// order a CTA's box spans the whole point set; sorted along a Morton curve and cut into tiles that
// never cross a coarse cell, every CTA's box is small. Sorting the sources as well, in chunks of
// the kernel's source tile with one bounding box each, lets a CTA skip every chunk whose box is
// beyond the distance at which the kernel value is exactly zero in the lane type.
#pragma once

#include <cuda_runtime.h>

struct gbk_ctx;

namespace gbk {

struct OrderView {
  const int *perm = nullptr;    // sorted position -> row
  const int2 *tiles = nullptr;  // targets: [begin, end) sorted positions per CTA
  const int *ntiles = nullptr;  // targets: number of tiles (device)
  long tile_bound = 0;          // targets: upper bound on the number of tiles (grid size)
  const double *boxes = nullptr;  // sources: lo[d], hi[d] per chunk of `chunk` sorted sources
};

// Target order for CTAs of `tile` targets; `sigma` sets the coarse cell width (in units of the
// FP32 coordinate scale) that no tile crosses. Kept in the context's target-order buffer until the
// next order_targets call on its stream.
int order_targets(gbk_ctx *c, int d, const double *x, long n, int tile, double sigma, OrderView *out);

// Source order with one bounding box per `chunk` consecutive sorted sources (the source-order
// buffer of the context).
int order_sources(gbk_ctx *c, int d, const double *y, long n, int chunk, OrderView *out);

// Copies narrays source arrays (row p of dst[k] = row perm[p] of src[k], cols[k] of its ld[k]
// columns) into the context's sorted-source buffer, one launch per array.
int gather_sources(gbk_ctx *c, const int *perm, long n, const double *const *src, const int *ld, const int *cols,
                   int narrays, double **dst);

// Own kernels launched by one order_targets / order_sources call (the radix sort is extra).
constexpr int kOrderTargetLaunches = 4;
constexpr int kOrderSourceLaunches = 4;

}  // namespace gbk
