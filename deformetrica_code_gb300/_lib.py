"""ctypes binding of libgbkernel.so (declared in include/gbk.h).

The library is the only compute path: if it is missing this module raises at import time.
There is no CPU or PyTorch fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# $GBK_LIBRARY selects another build of the same library (e.g. the bounds-checked one)
LIB_PATH = os.environ.get("GBK_LIBRARY") or os.path.join(HERE, "libgbkernel.so")

GBK_OK = 0
GBK_ERR_ARG = 1
GBK_ERR_UNSUPPORTED = 2
GBK_ERR_CUDA = 3
GBK_ERR_ALLOC = 4
GBK_ERR_TIMEOUT = 5
GBK_ERR_STATE = 6
GBK_ERR_BOUNDS = 7

GBK_MODE_F32C = 0
GBK_MODE_F64 = 1
GBK_ORDER_AUTO = 0
GBK_ORDER_OFF = 1
GBK_ORDER_SPATIAL = 2
GBK_ORDER_SPATIAL_NOPRUNE = 3
GBK_ORDER_TWO_FLOAT = 4
GBK_STAGING_AUTO = 0
GBK_STAGING_LOADS = 1
GBK_STAGING_BULK = 2
GBK_GRADIENT_REFERENCE = 0
GBK_GRADIENT_EXACT = 1
GBK_ESTIMATOR_FAST_GRADIENT_ASCENT = 0
GBK_ESTIMATOR_GRADIENT_ASCENT = 1

OPS = {
    "convolve": 0,
    "convolve_gradient_alpha_fused": 1,
    "gradient_alpha": 2,
    "gradient_varlin": 3,
    "gradient_dim": 4,
    "hessian": 5,
    "hessian_rowcol": 6,
    "special_hessian": 7,
}

_P = ctypes.c_void_p
_I = ctypes.c_int
_L = ctypes.c_long
_D = ctypes.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "gbk_version": (_I, []),
    "gbk_create": (_I, [_I, ctypes.POINTER(_P)]),
    "gbk_destroy": (None, [_P]),
    "gbk_last_error": (ctypes.c_char_p, [_P]),
    "gbk_set_stream": (_I, [_P, _P]),
    "gbk_get_stream": (_P, [_P]),
    "gbk_set_mode": (_I, [_P, _I]),
    "gbk_get_mode": (_I, [_P]),
    "gbk_evaluated_pairs": (ctypes.c_longlong, [_P]),
    "gbk_evaluated_pairs_by_op": (_I, [_P, ctypes.POINTER(ctypes.c_longlong), _I]),
    "gbk_set_order": (_I, [_P, _I]),
    "gbk_get_order": (_I, [_P]),
    "gbk_set_gradient_mode": (_I, [_P, _I]),
    "gbk_get_gradient_mode": (_I, [_P]),
    "gbk_set_estimator": (_I, [_P, _I]),
    "gbk_get_estimator": (_I, [_P]),
    "gbk_synchronize": (_I, [_P]),
    "gbk_launch_count": (ctypes.c_longlong, [_P]),
    "gbk_convolve": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P]),
    "gbk_convolve_gradient_alpha": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P, _P]),
    "gbk_convolve_and_gradient_alpha": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P, _P, _P]),
    "gbk_convolve_gradient": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P]),
    "gbk_convolve_gradient_dim": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _I, _P]),
    "gbk_convolve_gradient_kdp": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _I, _I, _P]),
    "gbk_convolve_hessian": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P]),
    "gbk_convolve_hessian_rowcol": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _I, _I, _P]),
    "gbk_convolve_hessian_kdpdq": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _I, _I, _I, _P]),
    "gbk_convolve_special_hessian": (_I, [_P, _I, _P, _P, _L, _D, _P, _P]),
    "gbk_forward_adjoint": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P, _P, _P, _P, _P]),
    "gbk_kernel_norm": (_I, [_P, _I, _I, _P, _P, _L, _D, _P]),
    "gbk_kernel_norm_noalloc": (_I, [_P, _I, _I, _P, _P, _L, _D, _P]),
    "gbk_autotune": (_I, [_P, _I, _I, _I, _L, _L, _D]),
    "gbk_autotune_data": (_I, [_P, _I, _I, _I, _P, _L, _P, _P, _L, _D, _P, ctypes.POINTER(_I), ctypes.POINTER(_I),
                               ctypes.POINTER(_D)]),
    "gbk_tune_save": (_I, [_P, ctypes.c_char_p]),
    "gbk_tune_load": (_I, [_P, ctypes.c_char_p]),
    "gbk_set_split": (_I, [_P, _I]),
    "gbk_shoot": (_I, [_P, _I, _L, _P, _P, _I, _D, _P, _P]),
    "gbk_flow_landmarks": (_I, [_P, _I, _L, _P, _P, _I, _D, _L, _P, _I, _P]),
    "gbk_adjoint_landmarks": (_I, [_P, _I, _L, _P, _P, _I, _D, _L, _P, _P, _I, _P]),
    "gbk_compute_update_at": (_I, [_P, _I, _L, _P, _P, _P, _P, _L, _P, _P, _D, _P, _P]),
    "gbk_adjoint_diffeo": (_I, [_P, _I, _L, _P, _P, _I, _D, _L, _P, _P, _I, _P, _P]),
    "gbk_currents_match": (_I, [_P, _L, _P, _L, _P, _L, _P, _L, _P, _D, _P, _P]),
    "gbk_varifold_match": (_I, [_P, _L, _P, _L, _P, _L, _P, _L, _P, _D, _P, _P]),
    "gbk_curve_currents_match": (_I, [_P, _I, _L, _P, _L, _P, _L, _P, _L, _P, _D, _P, _P]),
    "gbk_curve_varifold_match": (_I, [_P, _I, _L, _P, _L, _P, _L, _P, _L, _P, _D, _P, _P]),
    "gbk_pointcloud_match": (_I, [_P, _I, _L, _P, _P, _L, _P, _P, _D, _P, _P]),
    "gbk_volume_match": (_I, [_P, _I, _L, _P, _L, _P, _L, _P, _L, _P, _D, _P, _P]),
    "gbk_landmark_match": (_I, [_P, _I, _L, _P, _P, _P, _P]),
    "gbk_registration_set_point_weights": (_I, [_P, _P, _P]),
    "gbk_registration_create_multi": (_I, [_P, _I, _L, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _I, _D, _I,
                                           ctypes.POINTER(_P)]),
    "gbk_registration_set_template": (_I, [_P, _P]),
    "gbk_mo_atlas_create": (_I, [_P, _I, _L, _I, _P, _P, _P, _P, _P, _P, _P, _I, _P, _P, _P, _P, _I, _D, _I,
                                 ctypes.POINTER(_P)]),
    "gbk_mo_atlas_set_template_smoothing": (_I, [_P, _D]),
    "gbk_mo_atlas_set_lagged_template": (_I, [_P, _I]),
    "gbk_mo_atlas_step": (_I, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "gbk_mo_atlas_optimize": (_I, [_P, _P, _P, _P, _I, _I, _I, _D, _I, _D, _D, _D, _I, _P, _P, _P, _P, _P, _P, _P,
                                   _P, _P]),
    "gbk_mo_atlas_destroy": (None, [_P]),
    "gbk_geodesic_regression_create": (_I, [_P, _I, _L, _I, _P, _P, _P, _P, _P, _P, _P, _I, _P, _P, _P, _P, _P, _I, _D,
                                            _D, _D, _I, ctypes.POINTER(_P)]),
    "gbk_geodesic_regression_set_template_smoothing": (_I, [_P, _D]),
    "gbk_geodesic_regression_set_corrected_gradient": (_I, [_P, _I]),
    "gbk_geodesic_regression_set_graph": (_I, [_P, _I]),
    "gbk_geodesic_regression_step": (_I, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "gbk_geodesic_regression_optimize": (_I, [_P, _P, _P, _P, _I, _I, _I, _D, _I, _D, _D, _D, _I, _P, _P, _P, _P, _P,
                                              _P, _P, _P, _P]),
    "gbk_geodesic_regression_destroy": (None, [_P]),
    "gbk_p3m_convolve": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P, _D, _D, _P]),
    "gbk_p3m_convolve_gradient": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P, _D, _D, _P]),
    "gbk_p3m_convolve_gradient_alpha": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P, _P, _D, _D, _P]),
    "gbk_p3m_convolve_gradient_dim": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _I, _P, _D, _D, _P]),
    "gbk_p3m_convolve_hessian": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P, _D, _D, _P]),
    "gbk_p3m_convolve_hessian_rowcol": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _I, _I, _P, _D, _D, _P]),
    "gbk_p3m_convolve_gradient_kdp": (_I, [_P, _I, _I, _L, _L, _I, _I, _P]),
    "gbk_p3m_convolve_hessian_kdpdq": (_I, [_P, _I, _I, _L, _L, _I, _I, _I, _P]),
    "gbk_set_alloc_limit": (_I, [_P, ctypes.c_size_t]),
    "gbk_inject_pointer_device": (_I, [_P, _I]),
    "gbk_set_staging": (_I, [_P, _I]),
    "gbk_buffer_create": (_I, [_P, ctypes.POINTER(_P)]),
    "gbk_buffer_upload": (_I, [_P, _P, _P, ctypes.c_size_t]),
    "gbk_buffer_data": (_P, [_P]),
    "gbk_buffer_uploads": (ctypes.c_longlong, [_P]),
    "gbk_buffer_destroy": (None, [_P]),
    "gbk_get_staging": (_I, [_P]),
    "gbk_last_launch": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "gbk_image_points": (_I, [_P, _I, _P, _P, _P, _P]),
    "gbk_convolve_image_fast": (_I, [_P, _I, _P, _L, _P, _P, _L, _D, _P, _P, _P, _P]),
    "gbk_convolve_gradient_image_fast": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P, _P, _P, _P]),
    "gbk_convolve_gradient_image_fast_alpha": (_I, [_P, _I, _I, _P, _L, _P, _P, _L, _D, _P, _P, _P, _P, _P]),
    "gbk_flow_image_maps": (_I, [_P, _I, _L, _P, _P, _I, _D, _D, _I, _I, _P, _P, _P, _P, _P, _P]),
    "gbk_registration_create": (_I, [_P, _I, _L, _L, _P, _L, _P, _L, _P, _L, _P, _I, _D, _D, _D, _I, _I,
                                     ctypes.POINTER(_P)]),
    "gbk_registration_step": (_I, [_P, _P, _P, _P, _P, _P]),
    "gbk_registration_set_graph": (_I, [_P, _I]),
    "gbk_registration_trajectories": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "gbk_registration_graph_launches": (ctypes.c_longlong, [_P]),
    "gbk_registration_optimize": (_I, [_P, _P, _P, _I, _I, _D, _I, _D, _D, _D, _I, _P, _P, _P, _P, _P, _P, _P]),
    "gbk_registration_destroy": (None, [_P]),
    "gbk_atlas_create": (_I, [_P, _L, _P, _L, _P, _L, _P, _I, _P, _P, _P, _P, _I, _D, _D, _D, _I, _I,
                              ctypes.POINTER(_P)]),
    "gbk_atlas_step": (_I, [_P, _P, _P, _P, _P, _P]),
    "gbk_atlas_set_graph": (_I, [_P, _I]),
    "gbk_atlas_graph_launches": (ctypes.c_longlong, [_P]),
    "gbk_atlas_set_template_smoothing": (_I, [_P, _D]),
    "gbk_atlas_optimize": (_I, [_P, _P, _P, _P, _I, _I, _I, _D, _I, _D, _D, _D, _I, _P, _P, _P]),
    "gbk_atlas_destroy": (None, [_P]),
    "gbk_atlas_set_lagged_template": (_I, [_P, _I]),
}

_lib = None


def exported_symbols() -> list[str]:
    return sorted(SIGNATURES)


def load(path: str | None = None) -> ctypes.CDLL:
    """Loads libgbkernel.so and declares every signature. Raises if the library is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "(the CUDA library is the only implementation; there is no fallback)")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class GBKError(RuntimeError):
    """A failed library call (the reference throws std::runtime_error for the same cases)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[gbk error {code}] {msg}")
        self.code = code
