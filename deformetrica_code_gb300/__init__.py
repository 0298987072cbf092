"""GB300-native Gaussian kernel sums for Deformetrica (sm_103a CUDA behind a C ABI).

The compute path is libgbkernel.so (include/gbk.h). Importing this package loads it and raises
if it has not been built: there is no CPU or PyTorch fallback.
"""
from . import _lib
from ._lib import (GBKError, GBK_MODE_F32C, GBK_MODE_F64, GBK_ORDER_AUTO, GBK_ORDER_OFF, GBK_ORDER_SPATIAL,
                   GBK_ORDER_SPATIAL_NOPRUNE, GBK_ORDER_TWO_FLOAT, GBK_STAGING_AUTO, GBK_STAGING_LOADS, GBK_STAGING_BULK,
                   GBK_GRADIENT_REFERENCE, GBK_GRADIENT_EXACT,
                   GBK_ESTIMATOR_FAST_GRADIENT_ASCENT, GBK_ESTIMATOR_GRADIENT_ASCENT)

_lib.load()

from .kernel import (Context, GB300ExactKernel, GB300P3MKernel, p3m_convolve, p3m_convolve_gradient,  # noqa: E402
                     p3m_convolve_gradient_alpha, p3m_convolve_gradient_dim, p3m_convolve_hessian,
                     p3m_convolve_hessian_rowcol)
from .images import ImageGrid, flow_image_maps  # noqa: E402

__all__ = ["Context", "GB300ExactKernel", "GBKError", "GBK_MODE_F32C", "GBK_MODE_F64", "GBK_ORDER_AUTO",
           "GBK_ORDER_OFF", "GBK_ORDER_SPATIAL", "GBK_ORDER_SPATIAL_NOPRUNE", "GBK_ORDER_TWO_FLOAT", "GBK_STAGING_AUTO",
           "GBK_STAGING_LOADS", "GBK_STAGING_BULK",
           "GBK_GRADIENT_REFERENCE",
           "GBK_GRADIENT_EXACT", "GBK_ESTIMATOR_FAST_GRADIENT_ASCENT", "GBK_ESTIMATOR_GRADIENT_ASCENT", "p3m_convolve",
           "p3m_convolve_gradient", "p3m_convolve_gradient_alpha", "p3m_convolve_gradient_dim", "p3m_convolve_hessian",
           "p3m_convolve_hessian_rowcol", "GB300P3MKernel", "ImageGrid", "flow_image_maps"]
