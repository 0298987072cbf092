// Instantiations: Convolve, fused Convolve + alpha-gradient, alpha-gradient.
//
// FP32-compensated default (BLOCK threads, R targets per thread, TJ sources per tile, MERGE sources
// per compensated run, MINB CTAs per SM for the register allocator, UNR unroll of the source loop)
// and small shapes; the other shapes the autotuner chooses from are in gbk_k_conv_var.cu. Fused pass
// at N = M = 1e6 on GB300: default 564 ms; 2-way unroll 578 ms; 4 targets per thread at 2 CTAs/SM 603 ms; scalar FP32 lanes 568 ms;
// compensation terms in shared memory 605-636 ms (removed). Longer plain-FP32 runs before each
// compensated fold are faster but less accurate (spatial order, 1e6: MERGE 64 534 ms, normwise
// 1.9e-7; 128: 524 ms, 2.7e-7; 256: 519 ms, 4.0e-7), so every variant keeps runs of 64 and the
// autotuner only trades speed for speed. An expanded exponent, -|x'|^2 - |y'|^2 + 2 x'.y' with the
// two norms precomputed (two FP32 lane instructions fewer per pair, one more 16-byte shared load
// per source), measured 519 ms in every CTA (normwise error 9.8e-7: the expansion loses accuracy
// when the CTA's target box is wide) and 533 ms when restricted to CTAs whose box has a
// half-diagonal of at most one scaled unit, so the difference form stays. FP64 uses one target per
// thread. The two-float-coordinate variants are in gbk_k_conv_tf.cu.
#include "gbk_dispatch.h"

namespace gbk {

template <int D, int DV>
using OpCG = OpConvGradAlpha<D, DV, true>;
template <int D, int DV>
using OpGA = OpConvGradAlpha<D, DV, false>;

template <template <int, int> class OP>
constexpr int op_of() {
  return std::is_same<OP<3, 3>, OpConv<3, 3>>::value ? OP_CONV
         : std::is_same<OP<3, 3>, OpCG<3, 3>>::value ? OP_CONV_GRADA
                                                      : OP_GRADA;
}

template <template <int, int> class OP, int D, int DV>
static bool pick_conv_like(int mode, int variant, KernelEntry *e) {
  typedef OP<D, DV> O;
  if (mode == MODE_F64) {
    if (variant == VARIANT_SMALL) return set_entry<O, double, D, 64, 1, 32, 32, 8>(e);
    if (variant != 0) return false;
    return set_entry<O, double, D, 128, 1, 128, 128>(e);
  }
  if (variant == VARIANT_SMALL) return set_entry<O, float, D, 64, 2, 32, 32, 8>(e);
  if (variant != 0) return find_kernel_conv_shape(op_of<OP>(), D, DV, variant, e);
  // default: one float2 lane pair per thread, 4-way unrolled source loop, 3 CTAs of 256 per SM
  return set_entry<O, float, D, 256, 2, 256, 64, 3, 4>(e);
}


template <template <int, int> class OP>
static bool by_shape(int mode, int d, int dv, int variant, KernelEntry *e) {
  if (d == 2) {
    switch (dv) {
      case 1: return pick_conv_like<OP, 2, 1>(mode, variant, e);
      case 2: return pick_conv_like<OP, 2, 2>(mode, variant, e);
      case 3: return pick_conv_like<OP, 2, 3>(mode, variant, e);
      case 4: return pick_conv_like<OP, 2, 4>(mode, variant, e);
    }
  } else if (d == 3) {
    switch (dv) {
      case 1: return pick_conv_like<OP, 3, 1>(mode, variant, e);
      case 2: return pick_conv_like<OP, 3, 2>(mode, variant, e);
      case 3: return pick_conv_like<OP, 3, 3>(mode, variant, e);
      case 6: return pick_conv_like<OP, 3, 6>(mode, variant, e);
    }
  }
  return false;
}

bool find_kernel_conv(int op, int mode, int d, int dv, int variant, KernelEntry *e) {
  if (variant == VARIANT_TWO_FLOAT || variant == VARIANT_SMALL_TWO_FLOAT)
    return mode == MODE_F32C && find_kernel_conv_two_float(op, d, dv, variant, e);
  switch (op) {
    case OP_CONV: return by_shape<OpConv>(mode, d, dv, variant, e);
    case OP_CONV_GRADA: return by_shape<OpCG>(mode, d, dv, variant, e);
    case OP_GRADA: return by_shape<OpGA>(mode, d, dv, variant, e);
  }
  return false;
}

}  // namespace gbk
