// Instantiations: the warp-split kernels (gbk_pairs_warp.cuh) for kernel sums too small to fill the
// GPU in caller order -- Convolve, the fused Convolve + alpha-gradient and the alpha-gradient with
// one-float (VARIANT_WARP) and adaptive two-float (VARIANT_WARP_TWO_FLOAT) coordinates, and the fused
// control-point adjoint update (one-float). 8 warps (4 for the adjoint update, whose 15 accumulators
// fill the reduction area) share 64 targets, 2 per lane; registers capped for 2 CTAs per SM.
#include "gbk_dispatch.h"
#include "gbk_pairs_warp.cuh"

namespace gbk {

template <class O, typename T, int D>
static bool warp_entry(KernelEntry *e) {
  return set_entry_warp<O, T, D, 8, 2, 32, 2, 2>(e);  // KS, R, MERGE, UNR, MINB
}

template <template <int, int> class OP, typename T>
static bool by_shape_warp(int d, int dv, KernelEntry *e) {
  if (d == 2) {
    switch (dv) {
      case 1: return warp_entry<OP<2, 1>, T, 2>(e);
      case 2: return warp_entry<OP<2, 2>, T, 2>(e);
      case 3: return warp_entry<OP<2, 3>, T, 2>(e);
      case 4: return warp_entry<OP<2, 4>, T, 2>(e);
    }
  } else if (d == 3) {
    switch (dv) {
      case 1: return warp_entry<OP<3, 1>, T, 3>(e);
      case 2: return warp_entry<OP<3, 2>, T, 3>(e);
      case 3: return warp_entry<OP<3, 3>, T, 3>(e);
      case 6: return warp_entry<OP<3, 6>, T, 3>(e);
    }
  }
  return false;
}

template <int D, int DV>
using OpCGw = OpConvGradAlpha<D, DV, true>;
template <int D, int DV>
using OpGAw = OpConvGradAlpha<D, DV, false>;

template <typename T>
static bool by_op_warp(int op, int d, int dv, KernelEntry *e) {
  switch (op) {
    case OP_CONV: return by_shape_warp<OpConv, T>(d, dv, e);
    case OP_CONV_GRADA: return by_shape_warp<OpCGw, T>(d, dv, e);
    case OP_GRADA: return by_shape_warp<OpGAw, T>(d, dv, e);
  }
  return false;
}

bool find_kernel_warp(int op, int d, int dv, int variant, KernelEntry *e) {
  if (variant == VARIANT_WARP_TWO_FLOAT) return by_op_warp<f32w>(op, d, dv, e);
  if (variant != VARIANT_WARP) return false;
  if (op == OP_ADJCP) {
    if (dv != d) return false;
    if (d == 2) return set_entry_warp<OpAdjointCP<2>, float, 2, 4, 2, 32, 2, 2>(e);
    if (d == 3) return set_entry_warp<OpAdjointCP<3>, float, 3, 4, 2, 32, 2, 2>(e);
    return false;
  }
  return by_op_warp<float>(op, d, dv, e);
}

}  // namespace gbk
