"""Python front end of libppfr.so: the C ABI in include/pp_ops.h over torch
device tensors.

Field elements live in ``torch.int64`` tensors of shape ``(n, 4)`` (4 little-
endian 64-bit limbs, Montgomery form, canonical) on a CUDA device; the bytes
are exactly the reference's ``SyncedMemory`` contents.  Every call is enqueued
on the current torch stream.  There is no CPU fallback: without the compiled
library or a GPU every call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libppfr.so")

_lock = threading.Lock()
_lib = None

LDE_COEFFS, LDE_EVALS, LDE_SPREAD = 0, 1, 2


class PPError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(msg)
        self.status = status


def lib():
    """Load libppfr.so (build it with ppopp26-artifact_gb300/build.py)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError("libppfr.so is not built: run __graft_entry__.build()")
            L = ctypes.CDLL(LIB_PATH)
            v, u32, u64, i = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
            proto = {
                "pp_ntt": [v, v, u32, i, v],
                "pp_lde": [v, v, u32, u32, u32, v],
                "pp_gp_prefix": [v, u64, v],
                "pp_gp_perm": [v, v, v, v, u32, v],
                "pp_eval": [v, u64, v, v, v],
                "pp_div_xplusc": [v, u64, v, v],
                "pp_random_fr": [v, u64, u64, u64, v],
                "pp_ntt_prepare": [u32, i],
                "pp_release": [],
            }
            for name, args in proto.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = ctypes.c_int
            L.pp_last_error.restype = ctypes.c_char_p
            L.pp_last_error.argtypes = []
            L.pp_status_string.restype = ctypes.c_char_p
            L.pp_status_string.argtypes = [ctypes.c_int]
            L.pp_version.restype = ctypes.c_char_p
            L.pp_launch_count.restype = ctypes.c_uint64
            L.pp_launch_count.argtypes = []
            _lib = L
        return _lib


def check(status: int) -> None:
    if status != 0:
        L = lib()
        raise PPError(status, "%s: %s" % (L.pp_status_string(status).decode(),
                                          L.pp_last_error().decode()))


def _torch():
    import torch
    return torch


def _stream(stream=None):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t):
    assert t.is_cuda and t.is_contiguous() and t.dtype == _torch().int64, "need a contiguous int64 CUDA tensor"
    return ctypes.c_void_p(t.data_ptr())


def _lg(n: int) -> int:
    lg = n.bit_length() - 1
    if n <= 0 or (1 << lg) != n:
        raise ValueError("size must be a power of two, got %d" % n)
    return lg


def empty(n: int, device="cuda"):
    return _torch().empty((n, 4), dtype=_torch().int64, device=device)


def random_fr(n: int, seed: int, first_index: int = 0, device="cuda", stream=None):
    out = empty(n, device)
    check(lib().pp_random_fr(_ptr(out), n, seed & (2**64 - 1), first_index, _stream(stream)))
    return out


def ntt(x, inverse: bool = False, out=None, stream=None):
    lg = _lg(x.shape[0])
    if out is None:
        out = empty(x.shape[0], x.device)
    check(lib().pp_ntt(_ptr(x), _ptr(out), lg, int(inverse), _stream(stream)))
    return out


def intt(x, out=None, stream=None):
    return ntt(x, True, out, stream)


def lde(x, lam: int, mode: int = LDE_COEFFS, out=None, stream=None):
    lg = _lg(x.shape[0])
    if out is None:
        out = empty(x.shape[0] << lam, x.device)
    check(lib().pp_lde(_ptr(x), _ptr(out), lg, lam, mode, _stream(stream)))
    return out


def gp_prefix_(x, stream=None):
    """accumulate_mul_poly: exclusive prefix product, in place."""
    check(lib().pp_gp_prefix(_ptr(x), x.shape[0], _stream(stream)))
    return x


def gp_perm(w, sigma, params, out=None, stream=None):
    """Copy-constraint grand product z; params = (beta, gamma, k1, k2, k3) as a (5,4) tensor."""
    n = w[0].shape[0]
    lg = _lg(n)
    if out is None:
        out = empty(n, w[0].device)
    wp = (ctypes.c_void_p * 3)(*[t.data_ptr() for t in w])
    sp = (ctypes.c_void_p * 3)(*[t.data_ptr() for t in sigma])
    for t in list(w) + list(sigma):
        _ptr(t)
    check(lib().pp_gp_perm(ctypes.cast(wp, ctypes.c_void_p), ctypes.cast(sp, ctypes.c_void_p),
                           _ptr(params), _ptr(out), lg, _stream(stream)))
    return out


def evaluate(poly, x, out=None, stream=None):
    if out is None:
        out = empty(1, x.device)
    n = poly.shape[0]
    pp = _ptr(poly) if n else ctypes.c_void_p(0)
    check(lib().pp_eval(pp, n, _ptr(x), _ptr(out), _stream(stream)))
    return out


def div_xplusc_(p, c, stream=None):
    """poly_div_poly: quotient of p by (X + c), in place (top entry 0)."""
    check(lib().pp_div_xplusc(_ptr(p), p.shape[0], _ptr(c), _stream(stream)))
    return p


def prepare(lg_n: int, inverse: bool = False) -> None:
    check(lib().pp_ntt_prepare(lg_n, int(inverse)))


def launch_count() -> int:
    return int(lib().pp_launch_count())


def release() -> None:
    check(lib().pp_release())
