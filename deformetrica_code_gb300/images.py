"""The image grid of the kernel path: image geometry, pixel points, and the backward integration of
the image maps (the reference's Diffeos for image objects).

An image is its geometry: origin, spacing and size per axis with identity direction; its points are
listed first index fastest, as GridFunctions::ImageToPoints (src/support/utilities/
GridFunctions.cxx:41-60). GB300ExactKernel.ConvolveImageFast takes an ImageGrid.
"""
from __future__ import annotations

import ctypes

import numpy as np

from .kernel import Context, _check, _empty_like, _hptr, _ptr


class ImageGrid:
    """origin, spacing (physical units) and size (pixels) per axis; identity direction."""

    def __init__(self, origin, spacing, size):
        self.origin = np.ascontiguousarray(np.asarray(origin, dtype=np.float64).ravel())
        self.spacing = np.ascontiguousarray(np.asarray(spacing, dtype=np.float64).ravel())
        self.size = np.ascontiguousarray(np.asarray(size, dtype=np.int64).ravel())
        if not (len(self.origin) == len(self.spacing) == len(self.size)) or len(self.size) not in (2, 3):
            raise ValueError("origin, spacing and size need 2 or 3 entries each")
        if np.any(self.size <= 0) or np.any(self.spacing <= 0):
            raise ValueError("sizes and spacings must be positive")

    @property
    def d(self) -> int:
        return len(self.size)

    @property
    def pixels(self) -> int:
        return int(np.prod(self.size))

    def arrays(self, d: int):
        if d != self.d:
            raise ValueError(f"a {self.d}-D image for a {d}-D kernel")
        return self.origin, self.spacing, self.size

    def points(self, context: Context | None = None, device: bool = False):
        """The pixels' physical points (pixels x d), computed by gbk_image_points."""
        ctx = context or Context()
        if device:
            import torch
            out = torch.empty((self.pixels, self.d), dtype=torch.float64, device=f"cuda:{ctx.device}")
        else:
            out = np.empty((self.pixels, self.d))
        ctx.check(ctx.lib.gbk_image_points(ctx.h, self.d, _hptr(self.origin), _hptr(self.spacing), _hptr(self.size),
                                           _ptr(out)))
        return out


def flow_image_maps(pos_traj, mom_traj, sigma: float, image: ImageGrid, heun: bool = True, fast: bool = True,
                    bbox=None, span: float = 1.0, context: Context | None = None):
    """The reference's backward integration of the image maps (Diffeos.cxx:725-770) on the device:
    returns (maps T x pixels x d, stopped_at) with stopped_at the time index at which the bounding
    box (d x 2: lo, hi per axis) stopped it, or None. fast = True uses ConvolveImageFast's windowed
    sums, False the full kernel sums; both in the context's precision."""
    ctx = context or Context()
    d = image.d
    if pos_traj.ndim != 3 or pos_traj.shape[2] != d or mom_traj.shape != pos_traj.shape:
        raise ValueError("pos_traj and mom_traj: T x ncp x d each")
    T, ncp = pos_traj.shape[0], pos_traj.shape[1]
    pos2 = _check(pos_traj.reshape(T * ncp, d), "pos_traj", d)
    mom2 = _check(mom_traj.reshape(T * ncp, d), "mom_traj", d)
    maps = _empty_like(pos2, (T, image.pixels, d))
    box = None
    if bbox is not None:
        box = np.ascontiguousarray(np.asarray(bbox, dtype=np.float64).reshape(d, 2))
    stopped = ctypes.c_int(-1)
    ctx.bind_stream(pos2, mom2)
    ctx.check(ctx.lib.gbk_flow_image_maps(ctx.h, d, ncp, _ptr(pos2), _ptr(mom2), T, float(sigma), float(span),
                                          int(bool(heun)), int(bool(fast)), _hptr(image.origin),
                                          _hptr(image.spacing), _hptr(image.size),
                                          None if box is None else _hptr(box), _ptr(maps), ctypes.byref(stopped)))
    return maps, (None if stopped.value < 0 else stopped.value)
