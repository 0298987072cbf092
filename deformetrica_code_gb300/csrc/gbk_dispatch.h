// Host-side table of compiled kernel-sum kernels: (operation, precision, d, dv, variant) ->
// launcher. The instantiations live in gbk_k_conv.cu, gbk_k_grad.cu and gbk_k_hess.cu so that
// the build compiles them in parallel.
#pragma once

#include <cuda_runtime.h>

#include "gbk_pairs.cuh"

namespace gbk {

enum OpId {
  OP_CONV = 0,       // Convolve
  OP_CONV_GRADA = 1, // Convolve + ConvolveGradient(X, alpha), one pass
  OP_GRADA = 2,      // ConvolveGradient(X, alpha)
  OP_VARLIN = 3,     // ConvolveGradient(X)
  OP_GRADDIM = 4,    // ConvolveGradient(X, dim)   (p0 = dim)
  OP_HESSFULL = 5,   // ConvolveHessian(X)
  OP_HESSRC = 6,     // ConvolveHessian(X, row, col) (p0 = row, p1 = col)
  OP_SPECIAL = 7,    // ConvolveSpecialHessian(xi)
  OP_ADJCP = 8,      // control-point part of ComputeUpdateAt (fused)
  OP_COUNT = 9
};

// Launch-shape index for problems too small to fill the GPU with the default shape.
constexpr int VARIANT_SMALL = 8;
// Adaptive two-float coordinates (lane tag f32w), default and small shapes: compiled for the Convolve
// and alpha-gradient ops in FP32C mode; the automatic order's caller-order path below its size rule
// (gbk_ctx::plan).
constexpr int VARIANT_TWO_FLOAT = 9;
constexpr int VARIANT_SMALL_TWO_FLOAT = 10;
// Bulk asynchronous staging of the source tiles (lane tag f32b), default shape: compiled for the
// Convolve and alpha-gradient ops in FP32C mode, for the spatial order's sorted source copies.
constexpr int VARIANT_BULK = 11;
constexpr int VARIANT_BULK_128 = 12;  // the same with 128-thread CTAs and 128-source chunks
// Warp-split kernels (gbk_pairs_warp.cuh) for problems too small to fill the GPU, caller order with
// packed coordinates: one-float (Convolve-like ops and the fused control-point adjoint update) and
// adaptive two-float (Convolve-like ops), FP32C.
constexpr int VARIANT_WARP = 13;
constexpr int VARIANT_WARP_TWO_FLOAT = 14;

enum Mode { MODE_F32C = 0, MODE_F64 = 1 };

typedef cudaError_t (*LaunchFn)(PairArgs, int, cudaStream_t);
// batched: (args, items, nitems, reduce items, nreduce items, stream)
typedef cudaError_t (*LaunchBatchedFn)(const PairArgs *, const int4 *, int, const int2 *, int, cudaStream_t);

struct KernelEntry {
  LaunchFn fn;
  LaunchBatchedFn fnb;
  const void *kernel;  // the pair kernel (for occupancy queries)
  int block;  // threads per CTA
  int r;      // targets per thread
  int tj;     // sources per shared-memory tile
  int no;     // accumulators per target (partial-buffer width)
  int smem;   // dynamic shared memory bytes per CTA
  bool packable;  // reads packed coordinates in caller order (PairArgs::xp / yp; see packable)
  int tile;       // targets per CTA
  int ks;         // warps of a CTA dividing its sources (warp-split kernels), 0 otherwise
};

// Accumulators per target of an op (the partial buffer holds nsplit * no * nx doubles).
int op_outputs(int op, int d, int dv);

// Fills *e and returns true when the combination is compiled. dv must be one of the compiled
// column counts (see supported_dv); the host splits other counts into chunks.
bool find_kernel(int op, int mode, int d, int dv, int variant, KernelEntry *e);

// Compiled weight-column counts for dimension d, largest first (used to chunk any dv).
const int *supported_dv(int d, int *count);

// The allocation-free kernel norm's cached scratch address for `device` (current) is looked up
// again if it was cached (gbk_noalloc.cu); gbk_create calls it.
void noalloc_refresh_device(int device);

// Per-family lookups (one per instantiation file).
bool find_kernel_conv(int op, int mode, int d, int dv, int variant, KernelEntry *e);
bool find_kernel_conv_two_float(int op, int d, int dv, int variant, KernelEntry *e);
bool find_kernel_conv_bulk(int op, int d, int dv, int variant, KernelEntry *e);
bool find_kernel_conv_shape(int op, int d, int dv, int variant, KernelEntry *e);  // variants 1..4, FP32C
bool find_kernel_grad(int op, int mode, int d, int dv, int variant, KernelEntry *e);
bool find_kernel_hess(int op, int mode, int d, int dv, int variant, KernelEntry *e);
bool find_kernel_deform(int op, int mode, int d, int dv, int variant, KernelEntry *e);
bool find_kernel_warp(int op, int d, int dv, int variant, KernelEntry *e);  // VARIANT_WARP*, FP32C

}  // namespace gbk

namespace gbk {
// Helper for the instantiation files: records one compiled (op, T, D, BLOCK, R, TJ, MERGE) with
// MINB resident CTAs per SM requested from the register allocator, the per-source loop unrolled
// UNR times and the compensation terms in registers (CSM = 0) or shared memory (CSM = 1, 2).
template <class OpT, typename T, int D, int BLOCK, int R, int TJ, int MERGE, int MINB = 1, int UNR = 2,
          int CSM = 0>
inline bool set_entry(KernelEntry *e) {
  e->fn = &launch_pairs<OpT, T, D, BLOCK, R, TJ, MERGE, MINB, UNR, CSM>;
  e->fnb = &launch_pairs_batched<OpT, T, D, BLOCK, R, TJ, MERGE, MINB, UNR, CSM>;
  e->kernel = (const void *)&pair_kernel<OpT, T, D, BLOCK, R, TJ, MERGE, MINB, UNR, CSM>;
  e->block = BLOCK;
  e->r = R;
  e->tj = TJ;
  e->no = OpT::NO;
  e->smem = (int)pair_smem_bytes<OpT, T, D, BLOCK, R, TJ, CSM>();
  e->packable = packable<T, BLOCK>();
  e->tile = BLOCK * R;
  e->ks = 0;
  return true;
}
}  // namespace gbk
