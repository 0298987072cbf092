"""ctypes bindings to the FP64 oracle libraries (test infrastructure only).

Every function takes and returns row-major float64 numpy arrays, mirroring the reference's
``ExactKernel`` methods (file:line given per method in ``gauss_oracle.c``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_PORT_SRC = os.path.join(_HERE, "gauss_oracle.c")
_PORT_SO = os.path.join(_HERE, "_build", "liboracle_port.so")
_REF_SO = os.path.join(_HERE, "_ref", "libref_exactkernel.so")
_REF_SCRIPT = os.path.join(_HERE, "build_ref.sh")
_lock = threading.Lock()


def port_path() -> str:
    return _PORT_SO


def reference_path() -> str:
    return _REF_SO


def build_port(force: bool = False) -> str:
    """Compile gauss_oracle.c with gcc (-O2 -fopenmp, the reference's RELEASE level)."""
    with _lock:
        if (not force and os.path.exists(_PORT_SO)
                and os.path.getmtime(_PORT_SO) >= os.path.getmtime(_PORT_SRC)):
            return _PORT_SO
        os.makedirs(os.path.dirname(_PORT_SO), exist_ok=True)
        tmp = _PORT_SO + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-std=c11",
                               _PORT_SRC, "-o", tmp, "-lm"])
        os.replace(tmp, _PORT_SO)
        return _PORT_SO


REFERENCE_ENV = "DEFORMETRICA_REFERENCE_DIR"


def reference_root() -> str:
    """The reference's source tree for the recipes that read it (this package, the golden-fixture
    script, the binding tests): the directory named by $DEFORMETRICA_REFERENCE_DIR, else the
    checkout location of this build's container. Absent on machines without the tree."""
    return os.environ.get(REFERENCE_ENV) or "/root/reference"


def build_reference(reference_root: str | None = None) -> str | None:
    """Build oracle/_ref from the reference sources when they are present; else return None."""
    if reference_root is None:
        reference_root = globals()["reference_root"]()
    if not os.path.isdir(os.path.join(reference_root, "src", "support", "kernels")):
        return None
    with _lock:
        if not os.path.exists(_REF_SO):
            subprocess.check_call(["bash", _REF_SCRIPT, reference_root],
                                  stdout=subprocess.DEVNULL)
    return _REF_SO


_D = ctypes.POINTER(ctypes.c_double)
_L = ctypes.c_long
_I = ctypes.c_int
_F = ctypes.c_double

_SIGS = {
    "oracle_convolve": [_I, _I, _D, _L, _D, _D, _L, _F, _D],
    "oracle_grad_alpha": [_I, _I, _D, _L, _D, _D, _L, _F, _D, _D],
    "oracle_grad_varlin": [_I, _I, _D, _L, _D, _D, _L, _F, _D],
    "oracle_grad_dim": [_I, _I, _D, _L, _D, _D, _L, _F, _I, _D],
    "oracle_grad_kdp": [_I, _I, _D, _L, _D, _D, _L, _F, _I, _I, _D],
    "oracle_hess_full": [_I, _I, _D, _L, _D, _D, _L, _F, _D],
    "oracle_hess_rowcol": [_I, _I, _D, _L, _D, _D, _L, _F, _I, _I, _D],
    "oracle_hess_kdpdq": [_I, _I, _D, _L, _D, _D, _L, _F, _I, _I, _I, _D],
    "oracle_special_hessian": [_I, _I, _D, _D, _L, _F, _D, _D],
}
# exported by the reference library only: the image-grid methods through the ITK stand-ins
_REF_ONLY = {
    "oracle_ref_image_fast": [_I, _I, _I, _D, _L, _D, _D, _L, _F, _D, _D, _D, ctypes.POINTER(ctypes.c_long), _D],
    "oracle_ref_p3m": [_I, _I, _I, _D, _L, _D, _D, _L, _F, _D, _D, _D, _F, _F, _I, _I, _I, _D],
}
# exported by the port only (test denominators, no reference method)
_PORT_ONLY = {
    "oracle_convolve_mag": [_I, _I, _D, _L, _D, _D, _L, _F, _I, _D],
    "oracle_grad_alpha_mag": [_I, _I, _D, _L, _D, _D, _L, _F, _D, _I, _D],
}


def _c(a: np.ndarray):
    return a.ctypes.data_as(_D)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


class OracleError(RuntimeError):
    pass


class OracleLib:
    """One loaded oracle library (``port`` or ``reference``) with numpy-level methods."""

    def __init__(self, path: str, kind: str):
        self.kind = kind
        self.path = path
        self._lib = ctypes.CDLL(path)
        for name, argt in _SIGS.items():
            fn = getattr(self._lib, name)
            fn.argtypes = argt
            fn.restype = ctypes.c_int
        for name, argt in {**_PORT_ONLY, **_REF_ONLY}.items():
            if hasattr(self._lib, name):
                fn = getattr(self._lib, name)
                fn.argtypes = argt
                fn.restype = ctypes.c_int
        self._lib.oracle_last_error.restype = ctypes.c_char_p

    def _check(self, rc: int):
        if rc != 0:
            msg = self._lib.oracle_last_error().decode() if rc == -1 else "bad dimension"
            raise OracleError(msg)

    @staticmethod
    def _prep(x, y, w):
        x, y, w = _f64(x), _f64(y), _f64(w)
        if x.ndim != 2 or y.ndim != 2 or w.ndim != 2:
            raise ValueError("x, y and w must be 2-D")
        return x, y, w, x.shape[1], w.shape[1]

    def convolve(self, x, y, w, sigma):
        x, y, w, d, dv = self._prep(x, y, w)
        out = np.zeros((x.shape[0], dv))
        self._check(self._lib.oracle_convolve(d, dv, _c(x), x.shape[0], _c(y), _c(w), y.shape[0],
                                              sigma, _c(out)))
        return out

    def grad_alpha(self, x, y, w, sigma, alpha):
        x, y, w, d, dv = self._prep(x, y, w)
        alpha = _f64(alpha)
        out = np.zeros((x.shape[0], d))
        self._check(self._lib.oracle_grad_alpha(d, dv, _c(x), x.shape[0], _c(y), _c(w),
                                                y.shape[0], sigma, _c(alpha), _c(out)))
        return out

    def convolve_mag(self, x, y, w, sigma, cond: bool = True):
        """Sum over j of (1 + a_ij) K_ij |w_j| (cond) or K_ij |w_j|: the denominator of the
        condition-aware (or plain-magnitude) error of each convolve element; a_ij = |x_i - y_j|^2 / sigma^2."""
        x, y, w, d, dv = self._prep(x, y, w)
        out = np.zeros((x.shape[0], dv))
        self._check(self._lib.oracle_convolve_mag(d, dv, _c(x), x.shape[0], _c(y), _c(w), y.shape[0], sigma,
                                                  int(cond), _c(out)))
        return out

    def grad_alpha_mag(self, x, y, w, sigma, alpha, cond: bool = True):
        """The same for grad_alpha: (2/sigma^2) sum_j (1 + a_ij) K (|alpha_i|.|w_j|) |x_i - y_j|."""
        x, y, w, d, dv = self._prep(x, y, w)
        alpha = _f64(alpha)
        out = np.zeros((x.shape[0], d))
        self._check(self._lib.oracle_grad_alpha_mag(d, dv, _c(x), x.shape[0], _c(y), _c(w), y.shape[0], sigma,
                                                    _c(alpha), int(cond), _c(out)))
        return out

    def grad_varlin(self, x, y, w, sigma):
        x, y, w, d, dv = self._prep(x, y, w)
        out = np.zeros((x.shape[0], dv, d))
        self._check(self._lib.oracle_grad_varlin(d, dv, _c(x), x.shape[0], _c(y), _c(w),
                                                 y.shape[0], sigma, _c(out)))
        return out

    def grad_dim(self, x, y, w, sigma, dim):
        x, y, w, d, dv = self._prep(x, y, w)
        out = np.zeros((x.shape[0], dv))
        self._check(self._lib.oracle_grad_dim(d, dv, _c(x), x.shape[0], _c(y), _c(w),
                                              y.shape[0], sigma, dim, _c(out)))
        return out

    def grad_kdp(self, x, y, w, sigma, k, dp):
        x, y, w, d, dv = self._prep(x, y, w)
        out = np.zeros((y.shape[0],))
        self._check(self._lib.oracle_grad_kdp(d, dv, _c(x), x.shape[0], _c(y), _c(w),
                                              y.shape[0], sigma, k, dp, _c(out)))
        return out

    def hess_full(self, x, y, w, sigma):
        x, y, w, d, dv = self._prep(x, y, w)
        out = np.zeros((x.shape[0], dv, d, d))
        self._check(self._lib.oracle_hess_full(d, dv, _c(x), x.shape[0], _c(y), _c(w),
                                               y.shape[0], sigma, _c(out)))
        return out

    def hess_rowcol(self, x, y, w, sigma, row, col):
        x, y, w, d, dv = self._prep(x, y, w)
        out = np.zeros((x.shape[0], dv))
        self._check(self._lib.oracle_hess_rowcol(d, dv, _c(x), x.shape[0], _c(y), _c(w),
                                                 y.shape[0], sigma, row, col, _c(out)))
        return out

    def hess_kdpdq(self, x, y, w, sigma, k, dp, dq):
        x, y, w, d, dv = self._prep(x, y, w)
        out = np.zeros((x.shape[0],))
        self._check(self._lib.oracle_hess_kdpdq(d, dv, _c(x), x.shape[0], _c(y), _c(w),
                                                y.shape[0], sigma, k, dp, dq, _c(out)))
        return out

    def special_hessian(self, y, w, sigma, xi):
        y, w, xi = _f64(y), _f64(w), _f64(xi)
        d, dv = y.shape[1], w.shape[1]
        out = np.zeros((y.shape[0], d))
        self._check(self._lib.oracle_special_hessian(d, dv, _c(y), _c(w), y.shape[0], sigma,
                                                     _c(xi), _c(out)))
        return out

    def image_fast(self, kind: int, x, y, w, sigma, origin, spacing, size, alpha=None):
        """The reference's own image-grid methods (reference library only): kind 0 ConvolveImageFast
        (nx x d), 1 ConvolveGradientImageFast(X, image) (nx x dv x d), 2 ConvolveGradientImageFast(X,
        alpha, image) (nx x d); identity direction."""
        x, y, w, d, dv = self._prep(x, y, w)
        nx = x.shape[0]
        a = _f64(alpha) if alpha is not None else np.zeros((nx, dv))
        o, sp = _f64(origin), _f64(spacing)
        sz = np.ascontiguousarray(size, dtype=np.int64)
        shape = {0: (nx, d), 1: (nx, dv, d), 2: (nx, d)}[kind]
        out = np.zeros(shape)
        self._check(self._lib.oracle_ref_image_fast(d, kind, dv, _c(x), nx, _c(y), _c(w), y.shape[0], sigma, _c(a),
                                                    _c(o), _c(sp), sz.ctypes.data_as(ctypes.POINTER(ctypes.c_long)),
                                                    _c(out)))
        return out

    P3M_KINDS = {"convolve": 0, "gradient": 1, "gradient_alpha": 2, "gradient_dim": 3, "hessian": 4,
                 "hessian_rowcol": 5, "special_hessian": 6, "gradient_kdp": 7, "hessian_kdpdq": 8}

    def p3m(self, method: str, x, y, w, sigma, lo, hi, ratio: float = 0.2, padding: float = 3.0, alpha=None,
            args=(0, 0, 0)):
        """The reference's own P3MKernel<double, d> (reference library only), with data domain [lo, hi],
        working spacing ratio and padding factor, through the ITK stand-ins (direct DFTs). method: a key
        of P3M_KINDS; alpha is the alpha of ConvolveGradient(X, alpha) or the xi of
        ConvolveSpecialHessian (which ignores x); args are dim / (row, col) / (k, dp) / (k, dp, dq)."""
        kind = self.P3M_KINDS[method]
        x, y, w, d, dv = self._prep(x, y, w)
        nx, ny = x.shape[0], y.shape[0]
        a = _f64(alpha) if alpha is not None else np.zeros((max(nx, ny), max(dv, d)))
        shape = {0: (nx, dv), 1: (nx, dv, d), 2: (nx, d), 3: (nx, dv), 4: (nx, dv, d, d), 5: (nx, dv),
                 6: (ny, d), 7: (nx,), 8: (nx,)}[kind]
        out = np.zeros(shape)
        a0, a1, a2 = (list(args) + [0, 0, 0])[:3]
        self._check(self._lib.oracle_ref_p3m(d, kind, dv, _c(x), nx, _c(y), _c(w), ny, sigma, _c(a),
                                             _c(_f64(lo)), _c(_f64(hi)), ratio, padding, a0, a1, a2, _c(out)))
        return out

    # Source-side adjoint by symmetry of K (see oracle_fwd_adjoint in gauss_oracle.c).
    def fwd_adjoint(self, x, y, w, sigma, alpha):
        v = self.convolve(x, y, w, sigma)
        gx = self.grad_alpha(x, y, w, sigma, alpha)
        gw = self.convolve(y, x, alpha, sigma)
        gy = self.grad_alpha(y, x, alpha, sigma, w)
        return v, gx, gy, gw


_cache: dict[str, OracleLib] = {}


def load(kind: str = "port") -> OracleLib:
    """Load the ``port`` (always buildable) or the ``reference`` library (may be absent)."""
    if kind in _cache:
        return _cache[kind]
    if kind == "port":
        lib = OracleLib(build_port(), "port")
    elif kind == "reference":
        path = _REF_SO if os.path.exists(_REF_SO) else build_reference()
        if path is None or not os.path.exists(path):
            raise FileNotFoundError("reference oracle library not built (reference tree absent)")
        lib = OracleLib(path, "reference")
    else:
        raise ValueError(kind)
    _cache[kind] = lib
    return lib
