// Instantiations: ConvolveHessian (full and single entry) and the fused ConvolveSpecialHessian.
#include "gbk_dispatch.h"

namespace gbk {

template <template <int, int> class OP, int D, int DV>
static bool pick_one(int mode, int variant, KernelEntry *e) {
  typedef OP<D, DV> O;
  if (variant == VARIANT_SMALL) {
    if (mode == MODE_F64) return set_entry<O, double, D, 64, 1, 32, 32, 8>(e);
    return set_entry<O, float, D, 64, 2, 32, 32, 8>(e);
  }
  if (variant != 0) return false;  // the default and the small shape only
  if (mode == MODE_F64) return set_entry<O, double, D, 128, 1, 128, 128>(e);
  return set_entry<O, float, D, 256, 2, 256, 64, 2, 4>(e);
}

template <template <int, int> class OP>
static bool by_shape(int mode, int d, int dv, int variant, KernelEntry *e) {
  if (d == 2) {
    switch (dv) {
      case 1: return pick_one<OP, 2, 1>(mode, variant, e);
      case 2: return pick_one<OP, 2, 2>(mode, variant, e);
      case 3: return pick_one<OP, 2, 3>(mode, variant, e);
      case 4: return pick_one<OP, 2, 4>(mode, variant, e);
    }
  } else if (d == 3) {
    switch (dv) {
      case 1: return pick_one<OP, 3, 1>(mode, variant, e);
      case 2: return pick_one<OP, 3, 2>(mode, variant, e);
      case 3: return pick_one<OP, 3, 3>(mode, variant, e);
      case 6: return pick_one<OP, 3, 6>(mode, variant, e);
    }
  }
  return false;
}

template <int D, int DV>
using OpSH = OpSpecialHessian<D>;

bool find_kernel_hess(int op, int mode, int d, int dv, int variant, KernelEntry *e) {
  switch (op) {
    case OP_HESSFULL: return by_shape<OpHessFull>(mode, d, dv, variant, e);
    case OP_HESSRC: return by_shape<OpHessRowCol>(mode, d, dv, variant, e);
    case OP_SPECIAL:
      if (dv != d) return false;
      if (d == 2) return pick_one<OpSH, 2, 2>(mode, variant, e);
      if (d == 3) return pick_one<OpSH, 3, 3>(mode, variant, e);
      return false;
  }
  return false;
}

}  // namespace gbk
