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
TUNE_CACHE = os.path.join(HERE, "tune_gb300.json")

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
                "pp_ntt_host": [v, v, u32, i, v],
                "pp_ntt_host_many": [v, v, u32, u32, i, v],
                "pp_to_mont": [v, v, u64, v],
                "pp_msm_g1": [v, v, u64, v, v],
                "pp_msm_g1_window_bits": [u64],
                "pp_to_base": [v, v, u64, v],
                "pp_count_noncanonical": [v, u64, v, v],
                "pp_lde_host": [v, v, u32, u32, u32, v],
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
            # radix splits tuned on this GPU model (pp_tune_load ignores another GPU's file)
            if os.path.exists(TUNE_CACHE) and os.environ.get("PP_NO_TUNE_CACHE") is None:
                L.pp_tune_load.argtypes = [ctypes.c_char_p]
                L.pp_tune_load.restype = ctypes.c_int
                try:
                    L.pp_tune_load(TUNE_CACHE.encode())
                except OSError:
                    pass
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


def _hptr(t):
    assert (not t.is_cuda) and t.is_contiguous() and t.dtype == _torch().int64, \
        "need a contiguous int64 host tensor"
    return ctypes.c_void_p(t.data_ptr())


def empty_pinned(n: int):
    return _torch().empty((n, 4), dtype=_torch().int64, pin_memory=True)


def ntt_host(x, inverse: bool = False, out=None, stream=None):
    """Transform of a page-locked host tensor into a page-locked host tensor
    (pp_ntt_host).  Asynchronous: synchronise the stream before reading out."""
    lg = _lg(x.shape[0])
    if out is None:
        out = empty_pinned(x.shape[0])
    check(lib().pp_ntt_host(_hptr(x), _hptr(out), lg, int(inverse), _stream(stream)))
    return out


def ntt_host_many(xs, inverse: bool = False, outs=None, stream=None):
    """pp_ntt_host_many: transforms of equal-sized page-locked host tensors,
    copies of neighbouring ones overlapping the transforms.  Asynchronous:
    synchronise the stream before reading outs."""
    if outs is None:
        outs = [empty_pinned(x.shape[0]) for x in xs]
    assert len(outs) == len(xs)
    if not xs:
        return outs
    lg = _lg(xs[0].shape[0])
    assert all(x.shape[0] == xs[0].shape[0] and o.shape[0] == x.shape[0] for x, o in zip(xs, outs))
    ins = (ctypes.c_void_p * len(xs))(*[_hptr(x).value for x in xs])
    ous = (ctypes.c_void_p * len(xs))(*[_hptr(o).value for o in outs])
    check(lib().pp_ntt_host_many(ins, ous, len(xs), lg, int(inverse), _stream(stream)))
    return outs


def ntt_out_of_core(x, inverse: bool = False, out=None, scratch=None, stream=None):
    """pp_ntt_out_of_core: page-locked host input, output and scratch (three
    distinct buffers); device memory holds only small twiddle tables.
    Asynchronous: synchronise the stream before reading out."""
    lg = _lg(x.shape[0])
    if out is None:
        out = empty_pinned(x.shape[0])
    if scratch is None:
        scratch = empty_pinned(x.shape[0])
    L = lib()
    L.pp_ntt_out_of_core.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                     ctypes.c_int, ctypes.c_void_p]
    L.pp_ntt_out_of_core.restype = ctypes.c_int
    check(L.pp_ntt_out_of_core(_hptr(x), _hptr(out), _hptr(scratch), lg, int(inverse), _stream(stream)))
    return out


def lde_out_of_core(x, lam: int, mode: int = LDE_COEFFS, out=None, scratch=None, stream=None):
    """pp_lde_out_of_core: page-locked host input (2^lg), output and scratch
    (2^(lg + lam) each), three distinct buffers.  Asynchronous: synchronise the
    stream before reading out."""
    lg = _lg(x.shape[0])
    if out is None:
        out = empty_pinned(x.shape[0] << lam)
    if scratch is None:
        scratch = empty_pinned(x.shape[0] << lam)
    L = lib()
    L.pp_lde_out_of_core.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                     ctypes.c_uint32, ctypes.c_uint32, ctypes.c_void_p]
    L.pp_lde_out_of_core.restype = ctypes.c_int
    check(L.pp_lde_out_of_core(_hptr(x), _hptr(out), _hptr(scratch), lg, lam, mode, _stream(stream)))
    return out


def device_alloc_bytes() -> int:
    """Bytes of device memory this library has requested so far."""
    L = lib()
    L.pp_device_alloc_bytes.restype = ctypes.c_uint64
    return int(L.pp_device_alloc_bytes())


def lde_host(x, lam: int, mode: int = LDE_COEFFS, out=None, stream=None):
    """pp_lde_host: page-locked host input and output."""
    lg = _lg(x.shape[0])
    if out is None:
        out = empty_pinned(x.shape[0] << lam)
    check(lib().pp_lde_host(_hptr(x), _hptr(out), lg, lam, mode, _stream(stream)))
    return out


# ------------------------------------------------------------------------ G1
def msm_g1(points, scalars, out=None, stream=None):
    """pp_msm_g1: points (n, 12) int64 (affine x, y over Fq, Montgomery),
    scalars (n, 4) int64 (plain integers) -> (3, 6) int64 Jacobian point
    (x, y, 1), all zero for infinity."""
    torch = _torch()
    n = points.shape[0]
    assert scalars.shape[0] == n and points.shape[1] == 12 and scalars.shape[1] == 4
    assert points.is_contiguous() and scalars.is_contiguous()
    if out is None:
        out = torch.empty((3, 6), dtype=torch.int64, device=points.device)
    pp_, sp_ = (ctypes.c_void_p(points.data_ptr()), ctypes.c_void_p(scalars.data_ptr())) if n else (None, None)
    check(lib().pp_msm_g1(pp_, sp_, n, ctypes.c_void_p(out.data_ptr()), _stream(stream)))
    return out


FR_ADD, FR_SUB, FR_MUL, FR_DIV = 0, 1, 2, 3
FR_NEG, FR_INV = 0, 1


def _ew_proto(L):
    if not hasattr(L, "_ew_proto"):
        v, u32, u64 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64
        for name, args in (("pp_fr_binary", [u32, v, v, v, u64, ctypes.c_int, v]),
                           ("pp_fr_unary", [u32, v, v, u64, v]), ("pp_fr_pow", [v, v, u64, u64, v]),
                           ("pp_fr_powers", [v, v, u64, v]), ("pp_fr_fill", [v, v, u64, v])):
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L._ew_proto = True
    return L


def fr_binary(op: int, a, b, out=None, stream=None):
    """pp_fr_binary: a op b element-wise, or a op b[0] when b has one element
    (the reference's *_mod_scalar).  out may be a or b (the in-place forms)."""
    n = a.shape[0]
    scalar = b.shape[0] == 1 and n != 1
    assert scalar or b.shape[0] == n
    if out is None:
        out = empty(n, a.device)
    L = _ew_proto(lib())
    check(L.pp_fr_binary(op, _ptr(a) if n else None, _ptr(b), _ptr(out) if n else None, n, int(scalar),
                         _stream(stream)))
    return out


def fr_unary(op: int, a, out=None, stream=None):
    """pp_fr_unary: -a or 1 / a (0 for 0) element-wise."""
    n = a.shape[0]
    if out is None:
        out = empty(n, a.device)
    if n:
        check(_ew_proto(lib()).pp_fr_unary(op, _ptr(a), _ptr(out), n, _stream(stream)))
    return out


def fr_pow(a, exponent: int, out=None, stream=None):
    """pp_fr_pow: a^exponent element-wise (exponent < 2^64)."""
    n = a.shape[0]
    if out is None:
        out = empty(n, a.device)
    if n:
        check(_ew_proto(lib()).pp_fr_pow(_ptr(a), _ptr(out), n, exponent, _stream(stream)))
    return out


def fr_powers(x, n: int, out=None, stream=None):
    """pp_fr_powers (gen_sequence): [1, x, x^2, ..., x^(n-1)]."""
    if out is None:
        out = empty(n, x.device)
    if n:
        check(_ew_proto(lib()).pp_fr_powers(_ptr(x), _ptr(out), n, _stream(stream)))
    return out


def fr_fill(x, n: int, out=None, stream=None):
    """pp_fr_fill (repeat_to_poly): n copies of x."""
    if out is None:
        out = empty(n, x.device)
    if n:
        check(_ew_proto(lib()).pp_fr_fill(_ptr(x), _ptr(out), n, _stream(stream)))
    return out


def msm_window_bits(n: int) -> int:
    return int(lib().pp_msm_g1_window_bits(n))


def g1_mul_gen(scalars, out=None, stream=None):
    """pp_g1_mul_gen: scalars (n, 4) int64 plain integers -> (n, 12) int64
    affine points s_i G (all zero for infinity)."""
    torch = _torch()
    assert scalars.dim() == 2 and scalars.shape[1] == 4 and scalars.is_contiguous()
    n = scalars.shape[0]
    if out is None:
        out = torch.empty((n, 12), dtype=torch.int64, device=scalars.device)
    L = lib()
    L.pp_g1_mul_gen.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p]
    L.pp_g1_mul_gen.restype = ctypes.c_int
    if n:
        check(L.pp_g1_mul_gen(ctypes.c_void_p(scalars.data_ptr()), n, ctypes.c_void_p(out.data_ptr()),
                              _stream(stream)))
    return out


class MsmBases:
    """pp_msm_g1_bases_*: window tables of a fixed point set in HBM, for
    repeated MSMs over the same points (pp_msm_g1_fixed).  Same results as
    msm_g1 bit for bit."""

    def __init__(self, points, window_bits: int = 0, stream=None):
        L = lib()
        if not hasattr(L, "_bases_proto"):
            v = ctypes.c_void_p
            L.pp_msm_g1_bases_create.argtypes = [v, ctypes.c_uint64, ctypes.c_uint32, v, v]
            L.pp_msm_g1_bases_destroy.argtypes = [v]
            L.pp_msm_g1_bases_info.argtypes = [v, v, v, v]
            L.pp_msm_g1_fixed.argtypes = [v, v, v, v]
            for f in (L.pp_msm_g1_bases_create, L.pp_msm_g1_bases_destroy, L.pp_msm_g1_bases_info,
                      L.pp_msm_g1_fixed):
                f.restype = ctypes.c_int
            L._bases_proto = True
        assert points.dim() == 2 and points.shape[1] == 12 and points.is_contiguous()
        self.n = points.shape[0]
        self._h = ctypes.c_void_p(0)
        check(L.pp_msm_g1_bases_create(ctypes.c_void_p(points.data_ptr()), self.n, window_bits,
                                       ctypes.byref(self._h), _stream(stream)))
        n, c, nbytes = ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint64()
        check(L.pp_msm_g1_bases_info(self._h, ctypes.byref(n), ctypes.byref(c), ctypes.byref(nbytes)))
        self.window_bits, self.table_bytes = int(c.value), int(nbytes.value)
        self._device = points.device

    def msm(self, scalars, out=None, stream=None):
        """sum_i s_i P_i -> (3, 6) int64 Jacobian point (x, y, 1), all zero for infinity."""
        torch = _torch()
        assert scalars.shape == (self.n, 4) and scalars.is_contiguous()
        if out is None:
            out = torch.empty((3, 6), dtype=torch.int64, device=self._device)
        check(lib().pp_msm_g1_fixed(self._h, ctypes.c_void_p(scalars.data_ptr()),
                                    ctypes.c_void_p(out.data_ptr()), _stream(stream)))
        return out

    def close(self):
        if self._h:
            check(lib().pp_msm_g1_bases_destroy(self._h))
            self._h = ctypes.c_void_p(0)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# -------------------------------------------------------------- data formats
def read_raw(path: str, n: int = None, pinned: bool = True):
    """Raw file of 32-byte little-endian Montgomery elements (the reference's
    input.bin format) -> (n, 4) int64 host tensor, page-locked by default."""
    torch = _torch()
    import numpy as np
    a = np.fromfile(path, dtype=np.int64, count=-1 if n is None else 4 * n)
    if a.size % 4 or (n is not None and a.size != 4 * n):
        raise ValueError("%s: expected %s whole 32-byte elements" % (path, n if n is not None else "only"))
    t = torch.empty((a.size // 4, 4), dtype=torch.int64, pin_memory=pinned)
    t.copy_(torch.from_numpy(a.reshape(-1, 4)))
    return t


def write_raw(path: str, t) -> None:
    """(n, 4) int64 tensor (host or device) -> raw 32-byte element file."""
    t.detach().cpu().contiguous().numpy().tofile(path)


def to_mont(x, out=None, stream=None):
    """pp_to_mont: a -> a R mod r."""
    out = empty(x.shape[0], x.device) if out is None else out
    check(lib().pp_to_mont(_ptr(x), _ptr(out), x.shape[0], _stream(stream)))
    return out


def to_base(x, out=None, stream=None):
    """pp_to_base: a -> a R^-1 mod r."""
    out = empty(x.shape[0], x.device) if out is None else out
    check(lib().pp_to_base(_ptr(x), _ptr(out), x.shape[0], _stream(stream)))
    return out


def count_noncanonical(x, stream=None) -> int:
    """Number of elements >= r (synchronises the stream to read the count)."""
    torch = _torch()
    c = torch.zeros(1, dtype=torch.int64, device=x.device)
    check(lib().pp_count_noncanonical(_ptr(x), x.shape[0], ctypes.c_void_p(c.data_ptr()), _stream(stream)))
    return int(c.item())


# ------------------------------------------------------ quotient constraints
class PermQuotientArgs(ctypes.Structure):
    """pp_perm_quotient_args (include/pp_ops.h)."""
    _fields_ = [("x", ctypes.c_void_p), ("w", ctypes.c_void_p * 4), ("z", ctypes.c_void_p),
                ("z_next", ctypes.c_void_p), ("sigma", ctypes.c_void_p * 4), ("mod", ctypes.c_void_p),
                ("l1", ctypes.c_void_p), ("alpha", ctypes.c_void_p), ("beta", ctypes.c_void_p),
                ("gamma", ctypes.c_void_p), ("k", ctypes.c_void_p * 3), ("one", ctypes.c_void_p)]


# argument order of the reference's compute_gate_constraint_allmerge_cuda
GATE_VECTORS = ["a_val", "b_val", "c_val", "d_val", "a_next_eval", "b_next_eval", "d_next_eval",
                "q_m", "q_l", "q_r", "q_o", "q_4", "q_c", "q_hl", "q_hr", "q_h4", "q_arith",
                "range", "logic", "fixed_group_add", "variable_group_add", "pi_eval_8n"]
GATE_SCALARS = ["four", "one", "two", "three", "kappa_range", "kappa_sq_range", "kappa_cu_range",
                "range_challenge", "P_D", "nine", "kappa_cu_logic", "eighteen", "eightyone",
                "eightythree", "kappa_qu_logic", "logic_challenge", "P_A", "kappa_fb", "kappa_sq_fb",
                "kappa_cu_fb", "fb_challenge", "kappa_vb", "kappa_sq_vb", "vb_challenge"]


class GateArgs(ctypes.Structure):
    """pp_gate_args (include/pp_ops.h)."""
    _fields_ = [("v", ctypes.c_void_p * len(GATE_VECTORS)), ("s", ctypes.c_void_p * len(GATE_SCALARS)),
                ("sbox_alpha", ctypes.c_int64)]


def _opt(t):
    return None if t is None else _ptr(t).value


def _perm_args(x=None, w=None, z=None, z_next=None, sigma=None, mod=None, l1=None, alpha=None,
               beta=None, gamma=None, k=None, one=None):
    a = PermQuotientArgs()
    a.x, a.z, a.z_next, a.mod, a.l1 = _opt(x), _opt(z), _opt(z_next), _opt(mod), _opt(l1)
    a.alpha, a.beta, a.gamma, a.one = _opt(alpha), _opt(beta), _opt(gamma), _opt(one)
    for j in range(4):
        a.w[j] = _opt(w[j]) if w is not None else None
        a.sigma[j] = _opt(sigma[j]) if sigma is not None else None
    for j in range(3):
        a.k[j] = _opt(k[j]) if k is not None else None
    return a


def _perm_call(name, args, result, stream):
    fn = getattr(lib(), name)
    fn.argtypes = [ctypes.POINTER(PermQuotientArgs), ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]
    fn.restype = ctypes.c_int
    check(fn(ctypes.byref(args), _ptr(result), result.shape[0], _stream(stream)))
    return result


def quotient_identity(x, w, z, alpha, beta, gamma, k, out=None, stream=None):
    """pp_quotient_identity: (x b + w_l + g)(x b k1 + w_r + g)(x b k2 + w_o + g)(x b k3 + w_4 + g) z alpha."""
    out = empty(x.shape[0], x.device) if out is None else out
    return _perm_call("pp_quotient_identity",
                      _perm_args(x=x, w=w, z=z, alpha=alpha, beta=beta, gamma=gamma, k=k), out, stream)


def quotient_copy_(result, sigma, mod, w, z_next, alpha, beta, gamma, stream=None):
    """pp_quotient_copy, in place on result."""
    return _perm_call("pp_quotient_copy", _perm_args(sigma=sigma, mod=mod, w=w, z_next=z_next,
                                                     alpha=alpha, beta=beta, gamma=gamma), result, stream)


def quotient_term_one_(result, z, l1, one, stream=None):
    """pp_quotient_term_one, in place on result."""
    return _perm_call("pp_quotient_term_one", _perm_args(z=z, l1=l1, one=one), result, stream)


def quotient_permutation(x, w, z, z_next, sigma, mod, l1, alpha, beta, gamma, k, one, out=None,
                         stream=None):
    """pp_quotient_permutation: the three permutation terms in one pass."""
    out = empty(x.shape[0], x.device) if out is None else out
    return _perm_call("pp_quotient_permutation",
                      _perm_args(x=x, w=w, z=z, z_next=z_next, sigma=sigma, mod=mod, l1=l1, alpha=alpha,
                                 beta=beta, gamma=gamma, k=k, one=one), out, stream)


def gate_constraint(vectors: dict, scalars: dict, sbox_alpha: int, out=None, stream=None):
    """pp_gate_constraint; vectors / scalars keyed by the reference's argument names."""
    a = GateArgs()
    for j, name in enumerate(GATE_VECTORS):
        a.v[j] = _ptr(vectors[name]).value
    for j, name in enumerate(GATE_SCALARS):
        a.s[j] = _ptr(scalars[name]).value
    a.sbox_alpha = int(sbox_alpha)
    first = vectors[GATE_VECTORS[0]]
    out = empty(first.shape[0], first.device) if out is None else out
    L = lib()
    L.pp_gate_constraint.argtypes = [ctypes.POINTER(GateArgs), ctypes.c_void_p, ctypes.c_uint64,
                                     ctypes.c_void_p]
    L.pp_gate_constraint.restype = ctypes.c_int
    check(L.pp_gate_constraint(ctypes.byref(a), _ptr(out), out.shape[0], _stream(stream)))
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


# ------------------------------------------------------------------ tuning
def set_split(lg_n: int, bits=None) -> None:
    """Radix split of 2^lg_n (pass sizes in bits); None restores the default."""
    L = lib()
    L.pp_ntt_set_split.argtypes = [ctypes.c_uint32, ctypes.c_void_p]
    L.pp_ntt_set_split.restype = ctypes.c_int
    if bits is None:
        check(L.pp_ntt_set_split(lg_n, None))
    else:
        arr = (ctypes.c_uint32 * 5)(*(list(bits) + [0] * (5 - len(bits))))
        check(L.pp_ntt_set_split(lg_n, ctypes.cast(arr, ctypes.c_void_p)))


def get_split(lg_n: int):
    L = lib()
    L.pp_ntt_get_split.argtypes = [ctypes.c_uint32, ctypes.c_void_p]
    L.pp_ntt_get_split.restype = ctypes.c_int
    arr = (ctypes.c_uint32 * 4)()
    check(L.pp_ntt_get_split(lg_n, ctypes.cast(arr, ctypes.c_void_p)))
    return [int(v) for v in arr if v]


def autotune(lg_n: int, reps: int = 3):
    """Time every balanced split of 2^lg_n, keep the fastest; returns (bits, ms)."""
    L = lib()
    L.pp_ntt_autotune.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    L.pp_ntt_autotune.restype = ctypes.c_int
    arr = (ctypes.c_uint32 * 4)()
    ms = ctypes.c_float(0.0)
    check(L.pp_ntt_autotune(lg_n, reps, ctypes.cast(arr, ctypes.c_void_p), ctypes.byref(ms)))
    return [int(v) for v in arr if v], float(ms.value)


def tune_save(path: str) -> None:
    L = lib()
    L.pp_tune_save.argtypes = [ctypes.c_char_p]
    L.pp_tune_save.restype = ctypes.c_int
    check(L.pp_tune_save(path.encode()))


def tune_load(path: str) -> None:
    L = lib()
    L.pp_tune_load.argtypes = [ctypes.c_char_p]
    L.pp_tune_load.restype = ctypes.c_int
    check(L.pp_tune_load(path.encode()))


# ------------------------------------------------------------------- batch
JOB_NTT, JOB_INTT, JOB_LDE_COEFFS, JOB_LDE_EVALS, JOB_LDE_SPREAD, JOB_GP = range(6)


class _Job(ctypes.Structure):
    _fields_ = [("d_in", ctypes.c_void_p), ("d_out", ctypes.c_void_p), ("lg_n", ctypes.c_uint32),
                ("kind", ctypes.c_uint32), ("lam", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class Batch:
    """A batch plan over fixed buffers: jobs are (kind, x, out, lam) tuples."""

    def __init__(self, jobs):
        L = lib()
        L.pp_batch_create.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p)]
        L.pp_batch_create.restype = ctypes.c_int
        for name in ("pp_batch_run",):
            getattr(L, name).argtypes = [ctypes.c_void_p, ctypes.c_void_p]
            getattr(L, name).restype = ctypes.c_int
        L.pp_batch_capture.argtypes = [ctypes.c_void_p]
        L.pp_batch_capture.restype = ctypes.c_int
        L.pp_batch_destroy.argtypes = [ctypes.c_void_p]
        L.pp_batch_destroy.restype = ctypes.c_int
        L.pp_batch_info.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        L.pp_batch_info.restype = ctypes.c_int
        self._keep = []
        arr = (_Job * max(1, len(jobs)))()
        for i, (kind, x, out, lam) in enumerate(jobs):
            _ptr(x)
            _ptr(out)
            self._keep += [x, out]
            arr[i] = _Job(x.data_ptr(), out.data_ptr(), _lg(x.shape[0]), kind, lam, 0)
        self._h = ctypes.c_void_p()
        check(L.pp_batch_create(ctypes.cast(arr, ctypes.c_void_p), len(jobs), ctypes.byref(self._h)))

    def run(self, stream=None):
        check(lib().pp_batch_run(self._h, _stream(stream)))

    def capture(self):
        check(lib().pp_batch_capture(self._h))

    def info(self):
        la, le = ctypes.c_uint32(), ctypes.c_uint32()
        ti = ctypes.c_uint64()
        check(lib().pp_batch_info(self._h, ctypes.byref(la), ctypes.byref(ti), ctypes.byref(le)))
        return {"launches": la.value, "tiles": ti.value, "levels": le.value}

    def close(self):
        if self._h:
            check(lib().pp_batch_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------- serving
class _ServerConfig(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_uint64), ("slots", ctypes.c_uint32), ("min_lg", ctypes.c_uint32),
                ("max_lg", ctypes.c_uint32), ("lam", ctypes.c_uint32), ("max_queue", ctypes.c_uint32),
                ("max_inflight_mm", ctypes.c_uint64)]


class _Bundle(ctypes.Structure):
    _fields_ = [("lg_n", ctypes.c_uint32), ("lam", ctypes.c_uint32), ("seed", ctypes.c_uint64),
                ("h_inputs", ctypes.c_void_p), ("h_params", ctypes.c_void_p)]


class BundleResult(ctypes.Structure):
    _fields_ = [("ticket", ctypes.c_uint64), ("status", ctypes.c_int), ("latency_ms", ctypes.c_double),
                ("queue_ms", ctypes.c_double), ("d_lde", ctypes.c_void_p * 3), ("d_z", ctypes.c_void_p),
                ("d_quotient", ctypes.c_void_p), ("d_evals", ctypes.c_void_p), ("d_w", ctypes.c_void_p * 3),
                ("d_sigma", ctypes.c_void_p * 3), ("d_params", ctypes.c_void_p)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_uint64), ("queued", ctypes.c_uint64), ("budget_used", ctypes.c_uint64),
                ("budget_peak", ctypes.c_uint64), ("admitted_while_busy", ctypes.c_uint64),
                ("max_concurrent", ctypes.c_uint64), ("p50_ms", ctypes.c_double), ("p99_ms", ctypes.c_double),
                ("bundles_per_s", ctypes.c_double)]


def copy_to_host(dptr: int, n_elems: int):
    """n field elements at a device address -> numpy uint64 (n, 4)."""
    import numpy as np
    out = np.empty((n_elems, 4), dtype=np.uint64)
    L = lib()
    L.pp_copy_to_host.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64]
    L.pp_copy_to_host.restype = ctypes.c_int
    check(L.pp_copy_to_host(out.ctypes.data, dptr, n_elems * 32))
    return out


def bundle_work(lg_n: int, lam: int) -> int:
    """pp_bundle_work: the algorithmic Montgomery multiplies of one bundle."""
    L = lib()
    L.pp_bundle_work.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    L.pp_bundle_work.restype = ctypes.c_uint64
    return int(L.pp_bundle_work(lg_n, lam))


class Server:
    """Continuous-batching server for prover-round bundles (pp_server_*)."""

    def __init__(self, budget_bytes: int, slots: int, min_lg: int, max_lg: int, lam: int = 2, max_queue: int = 0,
                 max_inflight_mm: int = 0):
        L = lib()
        L.pp_server_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p)]
        L.pp_server_submit.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
        L.pp_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p]
        L.pp_server_release.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.pp_server_cancel.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        L.pp_server_get_stats.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.pp_server_reset_stats.argtypes = [ctypes.c_void_p]
        L.pp_server_destroy.argtypes = [ctypes.c_void_p]
        for n in ("pp_server_create", "pp_server_submit", "pp_server_wait", "pp_server_release",
                  "pp_server_cancel", "pp_server_get_stats", "pp_server_reset_stats", "pp_server_destroy"):
            getattr(L, n).restype = ctypes.c_int
        self.lam = lam
        cfg = _ServerConfig(budget_bytes, slots, min_lg, max_lg, lam, max_queue, max_inflight_mm)
        self._h = ctypes.c_void_p()
        check(L.pp_server_create(ctypes.byref(cfg), ctypes.byref(self._h)))

    def submit(self, lg_n: int, seed: int, h_inputs=None, h_params=None) -> int:
        b = _Bundle(lg_n, self.lam, seed & (2**64 - 1),
                    None if h_inputs is None else h_inputs.data_ptr(),
                    None if h_params is None else h_params.data_ptr())
        t = ctypes.c_uint64()
        check(lib().pp_server_submit(self._h, ctypes.byref(b), ctypes.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_ms: int = 60000) -> BundleResult:
        r = BundleResult()
        check(lib().pp_server_wait(self._h, ticket, timeout_ms, ctypes.byref(r)))
        return r

    def wait_status(self, ticket: int, timeout_ms: int) -> int:
        return lib().pp_server_wait(self._h, ticket, timeout_ms, None)

    def release(self, ticket: int) -> None:
        check(lib().pp_server_release(self._h, ticket))

    def cancel(self, ticket: int) -> int:
        return lib().pp_server_cancel(self._h, ticket)

    def stats(self) -> dict:
        s = ServerStats()
        check(lib().pp_server_get_stats(self._h, ctypes.byref(s)))
        return {f: getattr(s, f) for f, _ in ServerStats._fields_}

    def reset_stats(self) -> None:
        check(lib().pp_server_reset_stats(self._h))

    def close(self) -> None:
        if self._h:
            check(lib().pp_server_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
