"""GB300 multi-limb SDPA Newton-step library: Python mirror of the C ABI.

``libsdpg.so`` (built in-tree by ``build.py``) holds every kernel and the
solver; this module only loads it through ctypes and converts arguments.
There is no CPU fallback: if the library is missing, importing ``lib``
raises.  Number arrays use the library's own element layout (see
``include/sdpg.h``): a numpy ``uint32`` array of shape ``(count, limbs + 2)``
holding ``[e, s, m[0], ..., m[limbs-1]]`` per value, column-major for matrices.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libsdpg.so")

OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_SQRT = 0, 1, 2, 3, 4


class SdpgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sdpg error {code}: {msg}")
        self.code = code


_lib = None


def _setup(lib: ctypes.CDLL) -> ctypes.CDLL:
    c = ctypes
    vp, i, ll, ch = c.c_void_p, c.c_int, c.c_longlong, c.c_char
    sig = {
        "sdpg_last_error": (c.c_char_p, []),
        "sdpg_version": (i, []),
        "sdpg_limbs_for_precision": (i, [i]),
        "sdpg_ml_elem_bytes": (i, [i]),
        "sdpg_ml_parse": (i, [i, c.c_char_p, vp]),
        "sdpg_ml_format": (i, [i, vp, i, c.c_char_p, i]),
        "sdpg_ml_from_double": (i, [i, vp, ll, vp]),
        "sdpg_ml_to_double": (i, [i, vp, ll, vp]),
        "sdpg_ml_from_mpf": (i, [i, vp, ll, vp]),
        "sdpg_ml_to_mpf": (i, [i, vp, ll, vp]),
        "sdpg_ml_host_op": (i, [i, i, ll, vp, vp, vp]),
        "sdpg_rgemm": (i, [i, ch, ch, i, i, i, vp, vp, i, vp, i, vp, vp, i]),
        "sdpg_rgemm_device": (i, [i, ch, ch, i, i, i, vp, vp, i, vp, i, vp, vp, i, vp]),
    }
    for name, (res, args) in sig.items():
        if hasattr(lib, name):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
    return lib


def lib() -> ctypes.CDLL:
    """The loaded CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} not built: run build.py (no CPU fallback exists)")
        _lib = _setup(ctypes.CDLL(LIB_PATH))
    return _lib


def check(rc: int) -> int:
    if rc < 0:
        raise SdpgError(rc, lib().sdpg_last_error().decode())
    return rc


def limbs_for_precision(bits: int) -> int:
    return check(lib().sdpg_limbs_for_precision(bits))


def ml_empty(count: int, limbs: int) -> np.ndarray:
    return np.zeros((count, limbs + 2), dtype=np.uint32)


def ml_parse(texts, limbs: int) -> np.ndarray:
    """Decimal strings -> ml array (exact up to truncation at the format's precision)."""
    texts = list(texts)
    out = ml_empty(len(texts), limbs)
    for k, t in enumerate(texts):
        check(lib().sdpg_ml_parse(limbs, t.encode(), out[k].ctypes.data))
    return out


def ml_from_double(x, limbs: int) -> np.ndarray:
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).ravel())
    out = ml_empty(x.size, limbs)
    check(lib().sdpg_ml_from_double(limbs, x.ctypes.data, x.size, out.ctypes.data))
    return out


def ml_to_double(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a)
    limbs = a.shape[1] - 2
    out = np.zeros(a.shape[0], dtype=np.float64)
    check(lib().sdpg_ml_to_double(limbs, a.ctypes.data, a.shape[0], out.ctypes.data))
    return out


def ml_format(a: np.ndarray, digits: int = 17) -> list[str]:
    a = np.ascontiguousarray(a)
    limbs = a.shape[1] - 2
    buf = ctypes.create_string_buffer(digits + 32)
    res = []
    for k in range(a.shape[0]):
        check(lib().sdpg_ml_format(limbs, a[k].ctypes.data, digits, buf, len(buf)))
        res.append(buf.value.decode())
    return res


def ml_host_op(op: int, a: np.ndarray, b: np.ndarray | None = None) -> np.ndarray:
    a = np.ascontiguousarray(a)
    b = a if b is None else np.ascontiguousarray(b)
    limbs = a.shape[1] - 2
    out = np.empty_like(a)
    check(lib().sdpg_ml_host_op(limbs, op, a.shape[0], a.ctypes.data, b.ctypes.data, out.ctypes.data))
    return out


def rgemm(transa: str, transb: str, m: int, n: int, k: int, alpha: np.ndarray, A: np.ndarray, lda: int,
          B: np.ndarray, ldb: int, beta: np.ndarray, C: np.ndarray, ldc: int) -> np.ndarray:
    """``C = alpha op(A) op(B) + beta C`` on the GPU (Rgemm signature); returns the new C."""
    limbs = A.shape[1] - 2
    A = np.ascontiguousarray(A)
    B = np.ascontiguousarray(B)
    C = np.array(C, copy=True, order="C")
    alpha = np.ascontiguousarray(alpha).reshape(-1)
    beta = np.ascontiguousarray(beta).reshape(-1)
    check(lib().sdpg_rgemm(limbs, transa.encode(), transb.encode(), m, n, k, alpha.ctypes.data,
                           A.ctypes.data, lda, B.ctypes.data, ldb, beta.ctypes.data, C.ctypes.data, ldc))
    return C
