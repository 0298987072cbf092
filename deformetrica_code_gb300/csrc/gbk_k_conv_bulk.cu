// Instantiations: Convolve, fused Convolve + alpha-gradient and alpha-gradient with bulk asynchronous
// staging of the source tiles (lane tag f32b, FP32C mode only): in the spatial order, where the
// sources are the library's sorted copies, one thread fetches each visited chunk of TJ coordinates
// and weights with cp.async.bulk into the other half of a double buffer while the CTA works on the
// current tile (PairArgs::bulk); launched on caller arrays it stages with ordinary loads. Two shapes:
// the default one, 3 CTAs of 256 threads per SM (36 KiB of shared memory each at d = dv = 3), and
// 6 CTAs of 128 threads with 128-source chunks (VARIANT_BULK_128, for the autotuner: smaller CTAs
// balance the uneven tiles that pruning leaves at small kernel widths).
#include "gbk_dispatch.h"

namespace gbk {

template <template <int, int> class OP, int D, int DV>
static bool pick_bulk(int variant, KernelEntry *e) {
  if (variant == VARIANT_BULK_128) return set_entry<OP<D, DV>, f32b, D, 128, 2, 128, 64, 6, 4>(e);
  return set_entry<OP<D, DV>, f32b, D, 256, 2, 256, 64, 3, 4>(e);
}

template <int D, int DV>
using OpCGb = OpConvGradAlpha<D, DV, true>;
template <int D, int DV>
using OpGAb = OpConvGradAlpha<D, DV, false>;

template <template <int, int> class OP>
static bool by_shape_bulk(int d, int dv, int variant, KernelEntry *e) {
  if (d == 2) {
    switch (dv) {
      case 1: return pick_bulk<OP, 2, 1>(variant, e);
      case 2: return pick_bulk<OP, 2, 2>(variant, e);
      case 3: return pick_bulk<OP, 2, 3>(variant, e);
      case 4: return pick_bulk<OP, 2, 4>(variant, e);
    }
  } else if (d == 3) {
    switch (dv) {
      case 1: return pick_bulk<OP, 3, 1>(variant, e);
      case 2: return pick_bulk<OP, 3, 2>(variant, e);
      case 3: return pick_bulk<OP, 3, 3>(variant, e);
      case 6: return pick_bulk<OP, 3, 6>(variant, e);
    }
  }
  return false;
}

bool find_kernel_conv_bulk(int op, int d, int dv, int variant, KernelEntry *e) {
  switch (op) {
    case OP_CONV: return by_shape_bulk<OpConv>(d, dv, variant, e);
    case OP_CONV_GRADA: return by_shape_bulk<OpCGb>(d, dv, variant, e);
    case OP_GRADA: return by_shape_bulk<OpGAb>(d, dv, variant, e);
  }
  return false;
}

}  // namespace gbk
