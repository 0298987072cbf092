// Instantiations: the further FP32C launch shapes of Convolve, the fused Convolve + alpha-gradient and
// the alpha-gradient that the autotuner chooses from (gbk_autotune), beside the default and small
// shapes of gbk_k_conv.cu:
//   1: the source loop unrolled 2 times instead of 4 (every shape);
//   2: 4 targets per thread (two float2 lane groups) at 2 CTAs of 256 threads per SM ((3, 3), (2, 2));
//   3: scalar FP32 lanes instead of packed float2 ((3, 3), (2, 2));
//   4: CTAs of 128 threads with 128-source tiles, 6 per SM (every shape).
// All keep the default's arithmetic (runs of 64 sources per compensated fold), so a tuned choice
// changes the speed only.
#include "gbk_dispatch.h"

namespace gbk {

template <template <int, int> class OP, int D, int DV>
static bool pick_shape(int variant, KernelEntry *e) {
  typedef OP<D, DV> O;
  constexpr bool hot = (D == 3 && DV == 3) || (D == 2 && DV == 2);
  switch (variant) {
    case 1: return set_entry<O, float, D, 256, 2, 256, 64, 3, 2>(e);
    case 4: return set_entry<O, float, D, 128, 2, 128, 64, 6, 4>(e);
    default: break;
  }
  if constexpr (hot) {
    switch (variant) {
      case 2: return set_entry<O, float, D, 256, 4, 256, 64, 2, 2>(e);
      case 3: return set_entry<O, f32s, D, 256, 2, 256, 64, 3, 4>(e);
      default: break;
    }
  }
  return false;
}

template <int D, int DV>
using OpCGv = OpConvGradAlpha<D, DV, true>;
template <int D, int DV>
using OpGAv = OpConvGradAlpha<D, DV, false>;

template <template <int, int> class OP>
static bool by_shape_var(int d, int dv, int variant, KernelEntry *e) {
  if (d == 2) {
    switch (dv) {
      case 1: return pick_shape<OP, 2, 1>(variant, e);
      case 2: return pick_shape<OP, 2, 2>(variant, e);
      case 3: return pick_shape<OP, 2, 3>(variant, e);
      case 4: return pick_shape<OP, 2, 4>(variant, e);
    }
  } else if (d == 3) {
    switch (dv) {
      case 1: return pick_shape<OP, 3, 1>(variant, e);
      case 2: return pick_shape<OP, 3, 2>(variant, e);
      case 3: return pick_shape<OP, 3, 3>(variant, e);
      case 6: return pick_shape<OP, 3, 6>(variant, e);
    }
  }
  return false;
}

bool find_kernel_conv_shape(int op, int d, int dv, int variant, KernelEntry *e) {
  switch (op) {
    case OP_CONV: return by_shape_var<OpConv>(d, dv, variant, e);
    case OP_CONV_GRADA: return by_shape_var<OpCGv>(d, dv, variant, e);
    case OP_GRADA: return by_shape_var<OpGAv>(d, dv, variant, e);
  }
  return false;
}

}  // namespace gbk
