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

// Source arrays to copy into sorted order: src[0] must be the coordinates (d columns); row p of
// copy k is row perm[p] of src[k] (its first cols[k] of ld[k] columns), rows cols[k] wide.
struct SourceCopies {
  int na = 0;
  const double *src[3] = {nullptr, nullptr, nullptr};
  int ld[3] = {0, 0, 0};
  int cols[3] = {0, 0, 0};
  double *dst[3] = {nullptr, nullptr, nullptr};  // filled by order_sources
  // arrays only read, to find non-finite source values (rows perm[p], first chk_cols[k] of
  // chk_ld[k] columns): a chunk holding one is never pruned, as every pair term it feeds is NaN or
  // infinite in the reference's sums however small the kernel value
  const double *chk[3] = {nullptr, nullptr, nullptr};
  int chk_ld[3] = {0, 0, 0};
  int chk_cols[3] = {0, 0, 0};
};

// A point set in spatial order (device memory of the context, valid until the slot is reused).
struct SortedSet {
  const int *perm = nullptr;       // sorted position -> row
  const unsigned *keys = nullptr;  // sorted keys, key_bits wide (Morton keys or their top bits)
  const double *box = nullptr;     // lo[d], hi[d] of the set
  long n = 0;
  int key_bits = 0;
  int launches = 0;  // own kernels launched by the sort (0 when an earlier sort was reused)
};

struct OrderView {
  const int *perm = nullptr;    // sorted position -> row
  const int2 *tiles = nullptr;  // targets: [begin, end) sorted positions per CTA
  const int *ntiles = nullptr;  // targets: number of tiles (device)
  long tile_bound = 0;          // targets: upper bound on the number of tiles
  long grid = 0;                // targets: CTAs to launch (they loop over the tiles)
  const double *boxes = nullptr;  // sources: lo[d], hi[d] per chunk of `chunk` sorted sources
  double *copies[3] = {nullptr, nullptr, nullptr};  // sources: the sorted copies requested
  int launches = 0;             // own kernels launched to build it
};

// Largest coordinate extent of the union of two point sets (max over axes of the union box's
// width; 0 for empty or all-NaN sets): one box launch and a pinned read-back that waits for the stream.
int order_extent(gbk_ctx *c, int d, const double *x, long nx, const double *y, long ny, double *extent);

// Sorts n points (steps 1-3) into one of the context's two sort slots, or, inside an order-cache
// scope of the context, returns the sort of the same rows made earlier in the same API call.
int order_sort(gbk_ctx *c, int d, const double *x, long n, SortedSet *out);

// Target tiles of `tile` sorted targets for CTAs; `sigma` sets the coarse cell width (in units of
// the FP32 coordinate scale) that no tile crosses. Kept in the context's tile buffer until the next
// call on its stream.
int order_targets(gbk_ctx *c, int d, const SortedSet &s, int tile, double sigma, OrderView *out);

// One bounding box per `chunk` (a multiple of 32) consecutive sorted sources and the sorted copies
// `copies` asks for (the context's source-box and sorted-source buffers).
int order_sources(gbk_ctx *c, int d, const double *y, const SortedSet &s, int chunk, const SourceCopies &copies,
                  OrderView *out);

// If any of the n rows of x (d columns), a (lda columns), b (ldb), e (lde) holds a NaN or an
// infinity (null arrays skipped), every one of the nchunks source-chunk boxes becomes unbounded, so
// the launch that reads them prunes nothing. `flag` is device scratch; asynchronous on `st`.
cudaError_t unbound_boxes_if_nonfinite(cudaStream_t st, int d, const double *x, long n, const double *a, int lda,
                                       const double *b, int ldb, const double *e, int lde, unsigned *flag,
                                       double *boxes, long nchunks);

}  // namespace gbk
