// Instantiations: the fused control-point adjoint update (OpAdjointCP).
#include "gbk_dispatch.h"

namespace gbk {

template <int D>
static bool pick_adjcp(int mode, int variant, KernelEntry *e) {
  typedef OpAdjointCP<D> O;
  if (variant != 0 && variant != VARIANT_SMALL) return false;  // the default and the small shape only
  if (mode == MODE_F64) {
    if (variant == VARIANT_SMALL) return set_entry<O, double, D, 64, 1, 32, 32, 4>(e);
    return set_entry<O, double, D, 128, 1, 64, 64, 2>(e);
  }
  if (variant == VARIANT_SMALL) return set_entry<O, float, D, 64, 2, 32, 32, 4>(e);
  return set_entry<O, float, D, 128, 2, 128, 64, 2>(e);
}

bool find_kernel_deform(int op, int mode, int d, int dv, int variant, KernelEntry *e) {
  if (op != OP_ADJCP || dv != d) return false;
  if (d == 2) return pick_adjcp<2>(mode, variant, e);
  if (d == 3) return pick_adjcp<3>(mode, variant, e);
  return false;
}

}  // namespace gbk
