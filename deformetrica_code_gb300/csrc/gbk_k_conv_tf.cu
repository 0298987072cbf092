// Instantiations: Convolve, fused Convolve + alpha-gradient and alpha-gradient with adaptive two-float
// coordinates (lane tag f32w, FP32C mode only), in the default and the small launch shape. A CTA
// whose targets spread wider than kTwoFloatWidth scaled units runs the two-float loop (low parts:
// D more float2 registers per target pair and D more values per staged source), any other CTA the
// one-float loop of the default variant. The default shape keeps 3 CTAs of 256 threads per SM
// (registers capped at 80, so narrow CTAs run as fast as in the default variant) except for 6 weight
// columns, whose two-float loop would spill heavily there and runs at 2.
#include "gbk_dispatch.h"

namespace gbk {

template <template <int, int> class OP, int D, int DV>
static bool pick_two_float(int variant, KernelEntry *e) {
  typedef OP<D, DV> O;
  if (variant == VARIANT_SMALL_TWO_FLOAT) return set_entry<O, f32w, D, 64, 2, 32, 32, 8>(e);
  constexpr int MINB = DV >= 6 ? 2 : 3;
  return set_entry<O, f32w, D, 256, 2, 256, 64, MINB, 4>(e);
}

template <int D, int DV>
using OpCGtf = OpConvGradAlpha<D, DV, true>;
template <int D, int DV>
using OpGAtf = OpConvGradAlpha<D, DV, false>;

template <template <int, int> class OP>
static bool by_shape_tf(int d, int dv, int variant, KernelEntry *e) {
  if (d == 2) {
    switch (dv) {
      case 1: return pick_two_float<OP, 2, 1>(variant, e);
      case 2: return pick_two_float<OP, 2, 2>(variant, e);
      case 3: return pick_two_float<OP, 2, 3>(variant, e);
      case 4: return pick_two_float<OP, 2, 4>(variant, e);
    }
  } else if (d == 3) {
    switch (dv) {
      case 1: return pick_two_float<OP, 3, 1>(variant, e);
      case 2: return pick_two_float<OP, 3, 2>(variant, e);
      case 3: return pick_two_float<OP, 3, 3>(variant, e);
      case 6: return pick_two_float<OP, 3, 6>(variant, e);
    }
  }
  return false;
}

bool find_kernel_conv_two_float(int op, int d, int dv, int variant, KernelEntry *e) {
  if (variant != VARIANT_TWO_FLOAT && variant != VARIANT_SMALL_TWO_FLOAT) return false;
  switch (op) {
    case OP_CONV: return by_shape_tf<OpConv>(d, dv, variant, e);
    case OP_CONV_GRADA: return by_shape_tf<OpCGtf>(d, dv, variant, e);
    case OP_GRADA: return by_shape_tf<OpGAtf>(d, dv, variant, e);
  }
  return false;
}

}  // namespace gbk
