"""Python mirror of the reference's kernel-object interface over libgbkernel.so.

``GB300ExactKernel`` has the method names, argument meanings and error behaviour of
``AbstractKernel`` / ``ExactKernel`` (src/support/kernels/AbstractKernel.h:34-187,
src/support/kernels/ExactKernel.cxx) so tests and scripts read like the reference's own kernel
tests. Every method is one call into the CUDA library (include/gbk.h); there is no CPU path.

Arrays may be numpy float64 arrays (host; results come back as numpy) or CUDA float64 torch
tensors (device; the call is queued on torch's current stream and returns CUDA tensors).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import GBKError, GBK_MODE_F32C, GBK_MODE_F64

try:  # torch is only needed for device-resident arrays
    import torch
except Exception:  # pragma: no cover - torch is present in every supported setup
    torch = None


def _is_torch(a) -> bool:
    return torch is not None and isinstance(a, torch.Tensor)


def _check(a, name: str, cols: int | None = None):
    if a is None:
        return None
    if _is_torch(a):
        if a.dtype != torch.float64:
            raise TypeError(f"{name}: expected float64, got {a.dtype}")
        if not a.is_contiguous():
            raise ValueError(f"{name}: must be contiguous (row-major)")
    else:
        if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
            raise TypeError(f"{name}: expected a C-contiguous float64 numpy array")
    if a.ndim != 2:
        raise ValueError(f"{name}: expected a 2-D matrix, got shape {tuple(a.shape)}")
    if cols is not None and a.shape[1] != cols:
        raise ValueError(f"{name}: expected {cols} columns, got {a.shape[1]}")
    return a


def _ptr(a):
    if a is None:
        return None
    if _is_torch(a):
        return ctypes.c_void_p(a.data_ptr()) if a.numel() else None
    return ctypes.c_void_p(a.ctypes.data) if a.size else None


class Context:
    """Owns one gbk_ctx (device buffers, stream, precision mode, tuning table)."""

    def __init__(self, device: int = 0, mode: int = GBK_MODE_F32C):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        rc = self.lib.gbk_create(device, ctypes.byref(h))
        if rc != 0:
            raise GBKError(rc, self.lib.gbk_last_error(None).decode())
        self.h = h
        self.device = device
        self.set_mode(mode)

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbk_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, rc: int):
        if rc != 0:
            raise GBKError(rc, self.lib.gbk_last_error(self.h).decode())

    def set_mode(self, mode: int):
        self.check(self.lib.gbk_set_mode(self.h, mode))
        self.mode = mode

    def set_order(self, order: int):
        """GBK_ORDER_AUTO / OFF / SPATIAL / SPATIAL_NOPRUNE / TWO_FLOAT (include/gbk.h)."""
        self.check(self.lib.gbk_set_order(self.h, order))

    def get_order(self) -> int:
        return int(self.lib.gbk_get_order(self.h))

    def set_gradient_mode(self, mode: int):
        """GBK_GRADIENT_REFERENCE (the reference's point-cloud and volume-mesh gradient formulas,
        default) or GBK_GRADIENT_EXACT (the derivatives of their matches) (include/gbk.h)."""
        self.check(self.lib.gbk_set_gradient_mode(self.h, mode))

    def get_gradient_mode(self) -> int:
        return int(self.lib.gbk_get_gradient_mode(self.h))

    def set_estimator(self, estimator: int):
        """GBK_ESTIMATOR_FAST_GRADIENT_ASCENT (default) or GBK_ESTIMATOR_GRADIENT_ASCENT for the
        optimize() methods (include/gbk.h)."""
        self.check(self.lib.gbk_set_estimator(self.h, estimator))

    def get_estimator(self) -> int:
        return int(self.lib.gbk_get_estimator(self.h))

    def set_split(self, n: int):
        self.check(self.lib.gbk_set_split(self.h, n))

    def set_alloc_limit(self, nbytes: int):
        """Fault injection for tests: device-buffer growth beyond nbytes fails with GBK_ERR_ALLOC
        (0 lifts the limit)."""
        self.check(self.lib.gbk_set_alloc_limit(self.h, int(nbytes)))

    def set_staging(self, staging: int):
        """GBK_STAGING_AUTO / LOADS / BULK: how the spatial order stages source tiles (include/gbk.h)."""
        self.check(self.lib.gbk_set_staging(self.h, staging))

    def last_launch(self) -> tuple[int, int]:
        """(compiled variant, source splits) of the context's last kernel-sum launch."""
        v, n = ctypes.c_int(), ctypes.c_int()
        self.check(self.lib.gbk_last_launch(self.h, ctypes.byref(v), ctypes.byref(n)))
        return v.value, n.value

    def inject_pointer_device(self, device: int):
        """Fault injection for tests: device allocations passed from now on are treated as memory
        of GPU `device` (-1 turns it off), so the refusal of another GPU's memory can be tested on
        one GPU."""
        self.check(self.lib.gbk_inject_pointer_device(self.h, int(device)))

    def launch_count(self) -> int:
        return int(self.lib.gbk_launch_count(self.h))

    def evaluated_pairs(self) -> int:
        """(target, source) pairs evaluated so far (pruned source chunks excluded); waits."""
        v = int(self.lib.gbk_evaluated_pairs(self.h))
        if v < 0:
            raise GBKError(3, "gbk_evaluated_pairs failed")
        return v

    def evaluated_pairs_by_op(self) -> list[int]:
        """Pairs evaluated so far per operation (gbk_evaluated_pairs_by_op order); waits."""
        counts = (ctypes.c_longlong * 9)()
        self.check(self.lib.gbk_evaluated_pairs_by_op(self.h, counts, 9))
        return [int(v) for v in counts]

    def bind_stream(self, *arrays):
        """Queue on torch's current stream when any argument is a CUDA tensor."""
        if any(_is_torch(a) and a.is_cuda for a in arrays if a is not None):
            self.use_torch_stream()
        else:
            self.check(self.lib.gbk_set_stream(self.h, None))

    def use_torch_stream(self):
        """Queue later calls on torch's current CUDA stream. torch reports the legacy default
        stream as handle 0; the library reads NULL as "the context's own stream", so that case
        is passed as cudaStreamLegacy (0x1)."""
        s = torch.cuda.current_stream(self.device).cuda_stream or 1
        self.check(self.lib.gbk_set_stream(self.h, ctypes.c_void_p(s)))

    def synchronize(self):
        self.check(self.lib.gbk_synchronize(self.h))

    def autotune(self, op: str, d: int, dv: int, nx: int, ny: int, sigma: float):
        """Tunes `op` (a key of _lib.OPS) for calls of this size on synthetic inputs (gbk_autotune)."""
        self.check(self.lib.gbk_autotune(self.h, _lib.OPS[op], d, dv, nx, ny, sigma))

    def autotune_data(self, op: str, x, y, w, sigma: float, alpha=None):
        """Tunes `op` on these arrays through the path their call takes (gbk_autotune_data); returns
        (variant, nsplit, ms per launch) of the choice."""
        x = _check(x, "x")
        y = _check(y, "y", x.shape[1])
        w = _check(w, "w")
        if alpha is not None:
            alpha = _check(alpha, "alpha", w.shape[1])
        v, n, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        if any(_is_torch(a) and a.is_cuda for a in (x, y, w, alpha) if a is not None):
            self.use_torch_stream()
        self.check(self.lib.gbk_autotune_data(self.h, _lib.OPS[op], x.shape[1], w.shape[1], _ptr(x), x.shape[0],
                                              _ptr(y), _ptr(w), y.shape[0], sigma, _ptr(alpha), ctypes.byref(v),
                                              ctypes.byref(n), ctypes.byref(ms)))
        return v.value, n.value, ms.value

    def tune_save(self, path: str):
        self.check(self.lib.gbk_tune_save(self.h, path.encode()))

    def tune_load(self, path: str):
        self.check(self.lib.gbk_tune_load(self.h, path.encode()))


def _hptr(a: np.ndarray):
    """A host array's address for the C ABI's small host-side arguments."""
    return ctypes.c_void_p(a.ctypes.data)


def _empty_like(ref, shape):
    if _is_torch(ref):
        return torch.empty(shape, dtype=torch.float64, device=ref.device)
    return np.empty(shape, dtype=np.float64)


class GB300ExactKernel:
    """Gaussian kernel K(x, y) = exp(-|x-y|^2 / sigma^2) evaluated by the GB300 library.

    Mirrors ExactKernel<double, PointDim> (ExactKernel.h:34-194): SetKernelWidth clamps the
    width at 1e-10 (AbstractKernel.h:87-89); sources/weights count mismatches raise like the
    reference's std::runtime_error.
    """

    def __init__(self, point_dim: int, kernel_width: float = 1.0, context: Context | None = None,
                 mode: int | None = None):
        if point_dim not in (2, 3):
            raise ValueError("PointDim must be 2 or 3")
        self.d = point_dim
        self.ctx = context or Context()
        if mode is not None:
            self.ctx.set_mode(mode)
        self.m_Sources = None
        self.m_Weights = None
        self.SetKernelWidth(kernel_width)
        self.m_Modified = False

    # -- encapsulation (AbstractKernel.h:83-115) --
    def GetKernelWidth(self) -> float:
        return self.m_KernelWidth

    def SetKernelWidth(self, h: float):
        if h < 1e-10:
            h = 1e-10
        self.m_KernelWidth = float(h)
        self.m_Modified = True

    def GetSources(self):
        return self.m_Sources

    def SetSources(self, X):
        self.m_Sources = _check(X, "sources", self.d)
        self.m_Modified = True

    def GetWeights(self):
        return self.m_Weights

    def SetWeights(self, W):
        self.m_Weights = _check(W, "weights")
        self.m_Modified = True

    def Clone(self) -> "GB300ExactKernel":
        k = GB300ExactKernel(self.d, self.m_KernelWidth, self.ctx)
        k.m_Sources, k.m_Weights, k.m_Modified = self.m_Sources, self.m_Weights, self.m_Modified
        return k

    # -- helpers --
    def _yw(self):
        Y, W = self.m_Sources, self.m_Weights
        if Y is None or W is None:
            raise RuntimeError("sources and weights must be set")
        if Y.shape[0] != W.shape[0]:
            raise RuntimeError("Sources and weights count mismatch")
        return Y, W

    def _call(self, fn, *args):
        self.ctx.check(fn(self.ctx.h, *args))

    # -- convolutions --
    def Convolve(self, X):
        """ExactKernel::Convolve (ExactKernel.cxx:51-74)."""
        X = _check(X, "X", self.d)
        Y, W = self._yw()
        out = _empty_like(X, (X.shape[0], W.shape[1]))
        self.ctx.bind_stream(X, Y, W)
        self._call(self.ctx.lib.gbk_convolve, self.d, W.shape[1], _ptr(X), X.shape[0], _ptr(Y),
                   _ptr(W), Y.shape[0], self.m_KernelWidth, _ptr(out))
        return out

    def ConvolveGradient(self, X, *args):
        """Overloads of ExactKernel::ConvolveGradient:
        (X) varlin :166-202 -> (nx, dv, d); (X, alpha) :264-275 -> (nx, d);
        (X, dim) :294-323 -> (nx, dv); (X, k, dp) :325-363 -> (ny,)."""
        X = _check(X, "X", self.d)
        Y, W = self._yw()
        dv, lib = W.shape[1], self.ctx.lib
        if len(args) == 0:
            out = _empty_like(X, (X.shape[0], dv, self.d))
            self.ctx.bind_stream(X, Y, W)
            self._call(lib.gbk_convolve_gradient, self.d, dv, _ptr(X), X.shape[0], _ptr(Y), _ptr(W),
                       Y.shape[0], self.m_KernelWidth, _ptr(out))
            return out
        if len(args) == 1 and not isinstance(args[0], (int, np.integer)):
            alpha = _check(args[0], "alpha", dv)
            if alpha.shape[0] != X.shape[0]:
                raise RuntimeError("alpha must have one row per target")
            out = _empty_like(X, (X.shape[0], self.d))
            self.ctx.bind_stream(X, Y, W, alpha)
            self._call(lib.gbk_convolve_gradient_alpha, self.d, dv, _ptr(X), X.shape[0], _ptr(Y),
                       _ptr(W), Y.shape[0], self.m_KernelWidth, _ptr(alpha), _ptr(out))
            return out
        if len(args) == 1:
            out = _empty_like(X, (X.shape[0], dv))
            self.ctx.bind_stream(X, Y, W)
            self._call(lib.gbk_convolve_gradient_dim, self.d, dv, _ptr(X), X.shape[0], _ptr(Y),
                       _ptr(W), Y.shape[0], self.m_KernelWidth, int(args[0]), _ptr(out))
            return out
        if len(args) == 2:
            out = _empty_like(X, (Y.shape[0],))
            self.ctx.bind_stream(X, Y, W)
            self._call(lib.gbk_convolve_gradient_kdp, self.d, dv, _ptr(X), X.shape[0], _ptr(Y),
                       _ptr(W), Y.shape[0], self.m_KernelWidth, int(args[0]), int(args[1]), _ptr(out))
            return out
        raise TypeError("ConvolveGradient takes (X), (X, alpha), (X, dim) or (X, k, dp)")

    def ConvolveAndGradient(self, X, alpha):
        """Convolve(X) and ConvolveGradient(X, alpha) in one fused pass."""
        X = _check(X, "X", self.d)
        Y, W = self._yw()
        alpha = _check(alpha, "alpha", W.shape[1])
        v = _empty_like(X, (X.shape[0], W.shape[1]))
        g = _empty_like(X, (X.shape[0], self.d))
        self.ctx.bind_stream(X, Y, W, alpha)
        self._call(self.ctx.lib.gbk_convolve_and_gradient_alpha, self.d, W.shape[1], _ptr(X),
                   X.shape[0], _ptr(Y), _ptr(W), Y.shape[0], self.m_KernelWidth, _ptr(alpha),
                   _ptr(v), _ptr(g))
        return v, g

    def ConvolveHessian(self, X, *args):
        """Overloads of ExactKernel::ConvolveHessian:
        (X) :365-397 -> (nx, dv, d, d); (X, row, col) :399-428 -> (nx, dv);
        (X, k, dp, dq) :430-470 -> (nx,)."""
        X = _check(X, "X", self.d)
        Y, W = self._yw()
        dv, lib = W.shape[1], self.ctx.lib
        self.ctx.bind_stream(X, Y, W)
        if len(args) == 0:
            out = _empty_like(X, (X.shape[0], dv, self.d, self.d))
            self._call(lib.gbk_convolve_hessian, self.d, dv, _ptr(X), X.shape[0], _ptr(Y), _ptr(W),
                       Y.shape[0], self.m_KernelWidth, _ptr(out))
            return out
        if len(args) == 2:
            out = _empty_like(X, (X.shape[0], dv))
            self._call(lib.gbk_convolve_hessian_rowcol, self.d, dv, _ptr(X), X.shape[0], _ptr(Y),
                       _ptr(W), Y.shape[0], self.m_KernelWidth, int(args[0]), int(args[1]), _ptr(out))
            return out
        if len(args) == 3:
            out = _empty_like(X, (X.shape[0],))
            self._call(lib.gbk_convolve_hessian_kdpdq, self.d, dv, _ptr(X), X.shape[0], _ptr(Y),
                       _ptr(W), Y.shape[0], self.m_KernelWidth, int(args[0]), int(args[1]),
                       int(args[2]), _ptr(out))
            return out
        raise TypeError("ConvolveHessian takes (X), (X, row, col) or (X, k, dp, dq)")

    def ConvolveSpecialHessian(self, xi):
        """AbstractKernel::ConvolveSpecialHessian (AbstractKernel.cxx:22-88), which P3MKernel
        inherits: composed on the host, as the reference does, from ConvolveHessian(Y) and
        ConvolveHessian(Y, r, q) with the weights beta x xi[:, r] (and their pairs), each a device
        particle-mesh sum. Host arrays (N x PointDim)."""
        Y, beta = self._yw()
        Y, beta = np.asarray(Y.cpu() if _is_torch(Y) else Y), np.asarray(beta.cpu() if _is_torch(beta) else beta)
        xi = np.ascontiguousarray(np.asarray(xi.cpu() if _is_torch(xi) else xi, dtype=np.float64))
        d = self.d
        if beta.shape[1] != d:
            raise RuntimeError("ConvolveSpecialHessian needs weights with PointDim columns")
        if xi.shape != Y.shape:
            raise RuntimeError("Y and Xi count mismatch")
        n = Y.shape[0]
        kw = self._kw()
        ha = p3m_convolve_hessian(Y, Y, beta, self.m_KernelWidth, **kw)
        out = np.zeros((n, d))
        for i in range(n):
            aux = np.zeros((d, d))
            for dim in range(d):
                aux -= ha[i, dim] * beta[i, dim]
            out[i] = aux @ xi[i]
        H = np.zeros((n, d, d))
        for r in range(d):
            wd = np.ascontiguousarray(beta * xi[:, r:r + 1])
            H[:, r, :] += p3m_convolve_hessian_rowcol(Y, Y, wd, self.m_KernelWidth, r, r, **kw)
            for q in range(r + 1, d):
                wt = np.ascontiguousarray(np.concatenate([wd, beta * xi[:, q:q + 1]], axis=1))
                hrq = p3m_convolve_hessian_rowcol(Y, Y, wt, self.m_KernelWidth, r, q, **kw)
                H[:, q, :] += hrq[:, :d]
                H[:, r, :] += hrq[:, d:]
        return out + np.einsum("irc,ic->ir", H, beta)

    def ConvolveSpecialHessian(self, xi):
        """AbstractKernel::ConvolveSpecialHessian (AbstractKernel.cxx:22-88)."""
        Y, W = self._yw()
        if W.shape[1] != self.d:
            raise RuntimeError("ConvolveSpecialHessian needs weights with PointDim columns")
        xi = _check(xi, "xi", self.d)
        if xi.shape[0] != Y.shape[0]:
            raise RuntimeError("Y and Xi count mismatch")
        out = _empty_like(xi, (Y.shape[0], self.d))
        self.ctx.bind_stream(Y, W, xi)
        self._call(self.ctx.lib.gbk_convolve_special_hessian, self.d, _ptr(Y), _ptr(W), Y.shape[0],
                   self.m_KernelWidth, _ptr(xi), _ptr(out))
        return out

    def ConvolveImageFast(self, X, image):
        """ExactKernel::ConvolveImageFast (ExactKernel.cxx:76-129): the sum over each control point's
        window of int(6 sigma) pixels per axis around it. `image` is an ImageGrid (origin, spacing,
        size) and X holds one (deformed) point per pixel, first index fastest; weights need
        PointDim columns. Raises GBKError when a window misses the image."""
        X = _check(X, "X", self.d)
        Y, W = self._yw()
        if W.shape[1] != self.d:
            raise RuntimeError("ConvolveImageFast needs weights with PointDim columns")
        origin, spacing, size = image.arrays(self.d)
        if X.shape[0] != int(np.prod(size)):
            raise ValueError(f"X has {X.shape[0]} rows for an image of {int(np.prod(size))} pixels")
        out = _empty_like(X, (X.shape[0], self.d))
        self.ctx.bind_stream(X, Y, W)
        self._call(self.ctx.lib.gbk_convolve_image_fast, self.d, _ptr(X), X.shape[0], _ptr(Y), _ptr(W), Y.shape[0],
                   self.m_KernelWidth, _hptr(origin), _hptr(spacing), _hptr(size), _ptr(out))
        return out

    def ConvolveGradientImageFast(self, X, *args):
        """ExactKernel::ConvolveGradientImageFast, both overloads (ExactKernel.cxx:207-290):
        (X, image) -> (pixels x dv x d) kernel gradients summed over the control points' windows,
        (X, alpha, image) -> (pixels x d) their contraction G_p^T alpha_p. The same windows as
        ConvolveImageFast; any weight column count."""
        X = _check(X, "X", self.d)
        Y, W = self._yw()
        if len(args) == 1:
            alpha, image = None, args[0]
        elif len(args) == 2:
            alpha, image = _check(args[0], "alpha", W.shape[1]), args[1]
        else:
            raise TypeError("ConvolveGradientImageFast(X, image) or (X, alpha, image)")
        origin, spacing, size = image.arrays(self.d)
        if X.shape[0] != int(np.prod(size)):
            raise ValueError(f"X has {X.shape[0]} rows for an image of {int(np.prod(size))} pixels")
        if alpha is not None and alpha.shape[0] != X.shape[0]:
            raise RuntimeError("X and alpha count mismatch")
        dv = W.shape[1]
        if alpha is None:
            out = _empty_like(X, (X.shape[0], dv, self.d))
            self.ctx.bind_stream(X, Y, W)
            self._call(self.ctx.lib.gbk_convolve_gradient_image_fast, self.d, dv, _ptr(X), X.shape[0], _ptr(Y),
                       _ptr(W), Y.shape[0], self.m_KernelWidth, _hptr(origin), _hptr(spacing), _hptr(size), _ptr(out))
        else:
            out = _empty_like(X, (X.shape[0], self.d))
            self.ctx.bind_stream(X, Y, W, alpha)
            self._call(self.ctx.lib.gbk_convolve_gradient_image_fast_alpha, self.d, dv, _ptr(X), X.shape[0], _ptr(Y),
                       _ptr(W), Y.shape[0], self.m_KernelWidth, _ptr(alpha), _hptr(origin), _hptr(spacing),
                       _hptr(size), _ptr(out))
        return out

    def ForwardAdjoint(self, X, alpha):
        """Convolve plus the gradients of sum_i alpha_i . (K W)_i w.r.t. X, Y and W."""
        X = _check(X, "X", self.d)
        Y, W = self._yw()
        alpha = _check(alpha, "alpha", W.shape[1])
        v = _empty_like(X, (X.shape[0], W.shape[1]))
        gx = _empty_like(X, (X.shape[0], self.d))
        gy = _empty_like(X, (Y.shape[0], self.d))
        gw = _empty_like(X, (Y.shape[0], W.shape[1]))
        self.ctx.bind_stream(X, Y, W, alpha)
        self._call(self.ctx.lib.gbk_forward_adjoint, self.d, W.shape[1], _ptr(X), X.shape[0],
                   _ptr(Y), _ptr(W), Y.shape[0], self.m_KernelWidth, _ptr(alpha), _ptr(v), _ptr(gx),
                   _ptr(gy), _ptr(gw))
        return v, gx, gy, gw

    def KernelNorm(self):
        """<W, K W> over the sources, reduced in FP64 on the device."""
        Y, W = self._yw()
        out = np.zeros(1)
        self.ctx.bind_stream(Y, W)
        self._call(self.ctx.lib.gbk_kernel_norm, self.d, W.shape[1], _ptr(Y), _ptr(W), Y.shape[0],
                   self.m_KernelWidth, ctypes.c_void_p(out.ctypes.data))
        return float(out[0])


__all__ = ["Context", "GB300ExactKernel", "GBKError", "GBK_MODE_F32C", "GBK_MODE_F64"]


def _p3m(name, x, y, w, sigma, alpha, domain, spacing_ratio, padding_factor, out_cols, context, ints=()):
    ctx = context or Context()
    d = x.shape[1]
    _check(x, "x")
    _check(y, "y", d)
    _check(w, "w")
    if w.shape[0] != y.shape[0]:
        raise ValueError("sources and weights count mismatch")
    if alpha is not None:
        _check(alpha, "alpha", w.shape[1])
        if alpha.shape[0] != x.shape[0]:
            raise ValueError("alpha needs one row per target")
    dom = None if domain is None else np.ascontiguousarray(np.concatenate([np.asarray(domain[0], float).ravel(),
                                                                            np.asarray(domain[1], float).ravel()]))
    if dom is not None and dom.size != 2 * d:
        raise ValueError("domain: (lo[d], hi[d])")
    out = _empty_like(x, (x.shape[0],) + out_cols)
    ctx.bind_stream(x, y, w)
    args = [ctx.h, d, w.shape[1], _ptr(x), x.shape[0], _ptr(y), _ptr(w), y.shape[0], float(sigma)]
    if alpha is not None:
        args.append(_ptr(alpha))
    args += [int(v) for v in ints]
    args += [None if dom is None else ctypes.c_void_p(dom.ctypes.data), float(spacing_ratio), float(padding_factor),
             _ptr(out)]
    ctx.check(getattr(ctx.lib, name)(*args))
    return out


def p3m_convolve(x, y, w, sigma, domain=None, spacing_ratio: float = 0.2, padding_factor: float = 3.0,
                 context: Context | None = None):
    """The reference's P3MKernel::Convolve on the device (gbk_p3m_convolve): a particle-mesh
    approximation of sum_j K(x_i, y_j) w_j. domain = (lo, hi) or None for the bounding box of x, y."""
    return _p3m("gbk_p3m_convolve", x, y, w, sigma, None, domain, spacing_ratio, padding_factor, (w.shape[1],),
                context)


def p3m_convolve_gradient(x, y, w, sigma, domain=None, spacing_ratio: float = 0.2, padding_factor: float = 3.0,
                          context: Context | None = None):
    """P3MKernel::ConvolveGradient(X): nx x dv x d."""
    return _p3m("gbk_p3m_convolve_gradient", x, y, w, sigma, None, domain, spacing_ratio, padding_factor,
                (w.shape[1], x.shape[1]), context)


def p3m_convolve_gradient_alpha(x, y, w, sigma, alpha, domain=None, spacing_ratio: float = 0.2,
                                padding_factor: float = 3.0, context: Context | None = None):
    """P3MKernel::ConvolveGradient(X, alpha): nx x d."""
    return _p3m("gbk_p3m_convolve_gradient_alpha", x, y, w, sigma, alpha, domain, spacing_ratio, padding_factor,
                (x.shape[1],), context)


def p3m_convolve_gradient_dim(x, y, w, sigma, dim: int, domain=None, spacing_ratio: float = 0.2,
                              padding_factor: float = 3.0, context: Context | None = None):
    """P3MKernel::ConvolveGradient(X, dim): nx x dv."""
    return _p3m("gbk_p3m_convolve_gradient_dim", x, y, w, sigma, None, domain, spacing_ratio, padding_factor,
                (w.shape[1],), context, ints=(dim,))


def p3m_convolve_hessian(x, y, w, sigma, domain=None, spacing_ratio: float = 0.2, padding_factor: float = 3.0,
                         context: Context | None = None):
    """P3MKernel::ConvolveHessian(X): nx x dv x d x d."""
    return _p3m("gbk_p3m_convolve_hessian", x, y, w, sigma, None, domain, spacing_ratio, padding_factor,
                (w.shape[1], x.shape[1], x.shape[1]), context)


def p3m_convolve_hessian_rowcol(x, y, w, sigma, row: int, col: int, domain=None, spacing_ratio: float = 0.2,
                                padding_factor: float = 3.0, context: Context | None = None):
    """P3MKernel::ConvolveHessian(X, row, col): nx x dv."""
    return _p3m("gbk_p3m_convolve_hessian_rowcol", x, y, w, sigma, None, domain, spacing_ratio, padding_factor,
                (w.shape[1],), context, ints=(row, col))


class GB300P3MKernel:
    """The reference's P3MKernel<double, PointDim> (P3MKernel.h:32-286) on the device: the same
    method names and overloads as the exact kernel object, every sum a particle-mesh approximation
    (grid spacing = working_spacing_ratio x width, padding_factor x width of padding). The data
    domain is the bounding box of targets and sources unless set with SetDataDomain."""

    def __init__(self, point_dim: int, kernel_width: float = 1.0, context: Context | None = None,
                 working_spacing_ratio: float = 0.2, padding_factor: float = 3.0):
        if point_dim not in (2, 3):
            raise ValueError("PointDim must be 2 or 3")
        self.d = point_dim
        self.ctx = context or Context()
        self.ratio, self.padding = float(working_spacing_ratio), float(padding_factor)
        self.domain = None
        self.m_Sources = self.m_Weights = None
        self.SetKernelWidth(kernel_width)

    def SetKernelWidth(self, h: float):
        self.m_KernelWidth = float(max(h, 1e-10))

    def GetKernelWidth(self) -> float:
        return self.m_KernelWidth

    def SetSources(self, Y):
        self.m_Sources = _check(Y, "sources", self.d)

    def SetWeights(self, W):
        self.m_Weights = _check(W, "weights")

    def SetDataDomain(self, lo, hi):
        self.domain = (np.asarray(lo, float), np.asarray(hi, float))

    def _yw(self):
        Y, W = self.m_Sources, self.m_Weights
        if Y is None or W is None:
            raise RuntimeError("sources and weights must be set")
        if Y.shape[0] != W.shape[0]:
            raise RuntimeError("Sources and weights count mismatch")
        return Y, W

    def _kw(self):
        return dict(domain=self.domain, spacing_ratio=self.ratio, padding_factor=self.padding, context=self.ctx)

    def Convolve(self, X):
        Y, W = self._yw()
        return p3m_convolve(_check(X, "X", self.d), Y, W, self.m_KernelWidth, **self._kw())

    def ConvolveGradient(self, X, *args):
        """(X) -> (nx, dv, d); (X, alpha) -> (nx, d); (X, dim) -> (nx, dv); (X, k, dp) -> nx zeros,
        as the reference's stub."""
        X = _check(X, "X", self.d)
        Y, W = self._yw()
        if len(args) == 0:
            return p3m_convolve_gradient(X, Y, W, self.m_KernelWidth, **self._kw())
        if len(args) == 1 and not isinstance(args[0], (int, np.integer)):
            return p3m_convolve_gradient_alpha(X, Y, W, self.m_KernelWidth, args[0], **self._kw())
        if len(args) == 1:
            return p3m_convolve_gradient_dim(X, Y, W, self.m_KernelWidth, int(args[0]), **self._kw())
        if len(args) == 2:
            out = np.zeros(X.shape[0])
            self.ctx.check(self.ctx.lib.gbk_p3m_convolve_gradient_kdp(self.ctx.h, self.d, W.shape[1], X.shape[0],
                                                                      Y.shape[0], int(args[0]), int(args[1]),
                                                                      _hptr(out)))
            return out
        raise TypeError("ConvolveGradient takes (X), (X, alpha), (X, dim) or (X, k, dp)")

    def ConvolveHessian(self, X, *args):
        """(X) -> (nx, dv, d, d); (X, row, col) -> (nx, dv); (X, k, dp, dq) -> nx zeros, as the
        reference's stub."""
        X = _check(X, "X", self.d)
        Y, W = self._yw()
        if len(args) == 0:
            return p3m_convolve_hessian(X, Y, W, self.m_KernelWidth, **self._kw())
        if len(args) == 2:
            return p3m_convolve_hessian_rowcol(X, Y, W, self.m_KernelWidth, int(args[0]), int(args[1]), **self._kw())
        if len(args) == 3:
            out = np.zeros(X.shape[0])
            self.ctx.check(self.ctx.lib.gbk_p3m_convolve_hessian_kdpdq(self.ctx.h, self.d, W.shape[1], X.shape[0],
                                                                       Y.shape[0], int(args[0]), int(args[1]),
                                                                       int(args[2]), _hptr(out)))
            return out
        raise TypeError("ConvolveHessian takes (X), (X, row, col) or (X, k, dp, dq)")

    def ConvolveSpecialHessian(self, xi):
        """AbstractKernel::ConvolveSpecialHessian (AbstractKernel.cxx:22-88), which P3MKernel
        inherits: composed on the host, as the reference does, from ConvolveHessian(Y) and
        ConvolveHessian(Y, r, q) with the weights beta x xi[:, r] (and their pairs), each a device
        particle-mesh sum. Host arrays (N x PointDim)."""
        Y, beta = self._yw()
        Y, beta = np.asarray(Y.cpu() if _is_torch(Y) else Y), np.asarray(beta.cpu() if _is_torch(beta) else beta)
        xi = np.ascontiguousarray(np.asarray(xi.cpu() if _is_torch(xi) else xi, dtype=np.float64))
        d = self.d
        if beta.shape[1] != d:
            raise RuntimeError("ConvolveSpecialHessian needs weights with PointDim columns")
        if xi.shape != Y.shape:
            raise RuntimeError("Y and Xi count mismatch")
        n = Y.shape[0]
        kw = self._kw()
        ha = p3m_convolve_hessian(Y, Y, beta, self.m_KernelWidth, **kw)
        out = np.zeros((n, d))
        for i in range(n):
            aux = np.zeros((d, d))
            for dim in range(d):
                aux -= ha[i, dim] * beta[i, dim]
            out[i] = aux @ xi[i]
        H = np.zeros((n, d, d))
        for r in range(d):
            wd = np.ascontiguousarray(beta * xi[:, r:r + 1])
            H[:, r, :] += p3m_convolve_hessian_rowcol(Y, Y, wd, self.m_KernelWidth, r, r, **kw)
            for q in range(r + 1, d):
                wt = np.ascontiguousarray(np.concatenate([wd, beta * xi[:, q:q + 1]], axis=1))
                hrq = p3m_convolve_hessian_rowcol(Y, Y, wt, self.m_KernelWidth, r, q, **kw)
                H[:, q, :] += hrq[:, :d]
                H[:, r, :] += hrq[:, d:]
        return out + np.einsum("irc,ic->ir", H, beta)
