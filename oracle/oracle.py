"""ctypes front end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It wraps two libraries:

* ``oracle/build/libpporacle.so`` -- the C restatement in ``pp_oracle.c``
  (builds anywhere gcc is present, including the GPU host);
* ``oracle/_ref/libppref.so`` -- the reference's own CPU code for the path
  (blst field, ``naive_gp``/``naive_div`` from ``miss_ops.cu``), which only
  builds where the reference sources are checked out.

Arrays are numpy ``uint64`` of shape ``(n, 4)``: one row per Fr element, 4
little-endian limbs, Montgomery form (R = 2^256), canonical.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "libpporacle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libppref.so")
# the reference sources: $PP_REFERENCE_SRC, else the copy staged by
# ``make -C oracle stage REF_CHECKOUT=<checkout>``
REF_SRC = os.environ.get("PP_REFERENCE_SRC", os.path.join(HERE, "_ref", "src"))

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
RMONT = 1 << 256
ONE_MONT = RMONT % R

_lock = threading.Lock()
_lib = None
_ref = None
_ref_tried = False

_P = ctypes.POINTER(ctypes.c_uint64)


def _ptr(a: np.ndarray):
    assert a.dtype == np.uint64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_P)


def build(ref: bool | None = None) -> None:
    """Compile the oracle (and the reference harness when its sources exist)."""
    targets = ["all"]
    if ref is None:
        ref = os.path.isdir(REF_SRC)
    if ref:
        targets.append("ref")
    subprocess.run(["make", "-s", "-C", HERE, f"REF={REF_SRC}", "-j8", *targets], check=True,
                   stdout=subprocess.DEVNULL)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                subprocess.run(["make", "-s", "-C", HERE, "all"], check=True, stdout=subprocess.DEVNULL)
            L = ctypes.CDLL(LIB_PATH)
            v = ctypes.c_void_p
            i = ctypes.c_int
            u = ctypes.c_uint64
            sigs = {
                "or_fr_mul": [v, v, v], "or_fr_add": [v, v, v], "or_fr_sub": [v, v, v],
                "or_fr_neg": [v, v], "or_fr_pow": [v, v, v], "or_fr_inv": [v, v],
                "or_fr_to_mont": [v, v], "or_fr_from_mont": [v, v], "or_fr_one": [v],
                "or_root_of_unity": [i, i, v], "or_random_fr": [v, u, u, u],
                "or_ntt": [v, i, i, i], "or_lde_coeffs": [v, i, i, v, i],
                "or_lde_evals": [v, i, i, v, i], "or_lde_spread": [v, i, i, v, i],
                "or_gp_prefix": [v, u], "or_gp_perm": [v, v, v, v, v, i, v, i],
                "or_eval": [v, u, v, v, i], "or_div_xplusc": [v, u, v],
                "or_naive_gp": [v, u, v], "or_naive_div": [v, u, v, v],
                "or_first_diff": [v, v, u],
                "or_quotient_identity": [v, v, v, v, v, v, v, v, u],
                "or_quotient_copy": [v, v, v, v, v, v, v, v, u],
                "or_quotient_term_one": [v, v, v, v, u],
                "or_gate_constraint": [v, v, ctypes.c_int64, v, u],
                "or_g1_msm": [v, v, u, v, i], "or_g1_mul_gen": [v, u, v, i], "or_g1_add": [v, v, v],
            }
            for name, args in sigs.items():
                fn = getattr(L, name)
                fn.argtypes = args
                fn.restype = None
            L.or_naive_div.restype = ctypes.c_int
            L.or_first_diff.restype = ctypes.c_int64
            _lib = L
        return _lib


def ref_lib():
    """The reference's own CPU code, or None where it cannot be built."""
    global _ref, _ref_tried
    with _lock:
        if not _ref_tried:
            _ref_tried = True
            if not os.path.exists(REF_LIB_PATH) and os.path.isdir(REF_SRC):
                try:
                    subprocess.run(["make", "-s", "-C", HERE, f"REF={REF_SRC}", "-j8", "ref"],
                                   check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
                except (subprocess.CalledProcessError, OSError):
                    pass
            if os.path.exists(REF_LIB_PATH):
                L = ctypes.CDLL(REF_LIB_PATH)
                v = ctypes.c_void_p
                for name in ("ref_fr_mul", "ref_fr_add", "ref_fr_sub"):
                    getattr(L, name).argtypes = [v, v, v, ctypes.c_uint64]
                L.ref_fr_inv.argtypes = [v, v, ctypes.c_uint64]
                L.ref_naive_gp.argtypes = [ctypes.c_int, v, v]
                L.ref_naive_div.argtypes = [ctypes.c_int, v, v, v]
                _ref = L
        return _ref


# ------------------------------------------------------------------ helpers
def empty(n: int) -> np.ndarray:
    return np.empty((n, 4), dtype=np.uint64)


def to_int(row) -> int:
    return int(row[0]) | (int(row[1]) << 64) | (int(row[2]) << 128) | (int(row[3]) << 192)


def from_int(x: int) -> np.ndarray:
    return np.array([(x >> (64 * k)) & 0xFFFFFFFFFFFFFFFF for k in range(4)], dtype=np.uint64)


def mont(x: int) -> np.ndarray:
    """Montgomery representation of the integer x."""
    return from_int((x % R) * RMONT % R)


def unmont(row) -> int:
    return to_int(row) * pow(RMONT, -1, R) % R


def random_fr(n: int, seed: int, first_index: int = 0) -> np.ndarray:
    out = empty(n)
    if n:
        lib().or_random_fr(out.ctypes.data, n, seed & (2**64 - 1), first_index)
    return out


def _scalar(x) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(x, dtype=np.uint64).reshape(4))
    return a


def fr_mul(a, b):
    a, b, o = _scalar(a), _scalar(b), np.empty(4, np.uint64)
    lib().or_fr_mul(a.ctypes.data, b.ctypes.data, o.ctypes.data)
    return o


def fr_add(a, b):
    a, b, o = _scalar(a), _scalar(b), np.empty(4, np.uint64)
    lib().or_fr_add(a.ctypes.data, b.ctypes.data, o.ctypes.data)
    return o


def fr_sub(a, b):
    a, b, o = _scalar(a), _scalar(b), np.empty(4, np.uint64)
    lib().or_fr_sub(a.ctypes.data, b.ctypes.data, o.ctypes.data)
    return o


def fr_neg(a):
    a, o = _scalar(a), np.empty(4, np.uint64)
    lib().or_fr_neg(a.ctypes.data, o.ctypes.data)
    return o


def fr_inv(a):
    a, o = _scalar(a), np.empty(4, np.uint64)
    lib().or_fr_inv(a.ctypes.data, o.ctypes.data)
    return o


def fr_pow(a, e: int) -> np.ndarray:
    """a^e for an integer exponent 0 <= e < 2^256."""
    a = _scalar(a)
    ev = from_int(e)
    o = np.empty(4, np.uint64)
    lib().or_fr_pow(a.ctypes.data, ev.ctypes.data, o.ctypes.data)
    return o


def root_of_unity(lg: int, inverse: bool = False) -> np.ndarray:
    o = np.empty(4, np.uint64)
    lib().or_root_of_unity(lg, int(inverse), o.ctypes.data)
    return o


def ntt(a: np.ndarray, inverse: bool = False, nthreads: int = 0) -> np.ndarray:
    out = np.ascontiguousarray(a, dtype=np.uint64).copy()
    n = out.shape[0]
    lg = n.bit_length() - 1
    assert n == 1 << lg
    lib().or_ntt(out.ctypes.data, lg, int(inverse), nthreads)
    return out


def lde_coeffs(a: np.ndarray, lam: int, nthreads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64)
    n = a.shape[0]
    lg = n.bit_length() - 1
    out = empty(n << lam)
    lib().or_lde_coeffs(a.ctypes.data, lg, lam, out.ctypes.data, nthreads)
    return out


def lde_evals(a: np.ndarray, lam: int, nthreads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64)
    n = a.shape[0]
    lg = n.bit_length() - 1
    out = empty(n << lam)
    lib().or_lde_evals(a.ctypes.data, lg, lam, out.ctypes.data, nthreads)
    return out


def lde_spread(a: np.ndarray, lam: int, nthreads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64)
    n = a.shape[0]
    lg = n.bit_length() - 1
    out = empty(n << lam)
    lib().or_lde_spread(a.ctypes.data, lg, lam, out.ctypes.data, nthreads)
    return out


def gp_prefix(a: np.ndarray) -> np.ndarray:
    out = np.ascontiguousarray(a, dtype=np.uint64).copy()
    lib().or_gp_prefix(out.ctypes.data, out.shape[0])
    return out


def gp_perm(w, sigma, beta, gamma, ks, nthreads: int = 0) -> np.ndarray:
    w = [np.ascontiguousarray(x, dtype=np.uint64) for x in w]
    sigma = [np.ascontiguousarray(x, dtype=np.uint64) for x in sigma]
    n = w[0].shape[0]
    lg = n.bit_length() - 1
    assert n == 1 << lg
    wp = (ctypes.c_void_p * 3)(*[x.ctypes.data for x in w])
    sp = (ctypes.c_void_p * 3)(*[x.ctypes.data for x in sigma])
    k = np.ascontiguousarray(np.asarray(ks, dtype=np.uint64).reshape(3, 4))
    b, g = _scalar(beta), _scalar(gamma)
    z = empty(n)
    lib().or_gp_perm(ctypes.cast(wp, ctypes.c_void_p), ctypes.cast(sp, ctypes.c_void_p), b.ctypes.data,
                     g.ctypes.data, k.ctypes.data, lg, z.ctypes.data, nthreads)
    return z


def evaluate(poly: np.ndarray, x, nthreads: int = 0) -> np.ndarray:
    poly = np.ascontiguousarray(poly, dtype=np.uint64)
    xs, y = _scalar(x), np.empty(4, np.uint64)
    lib().or_eval(poly.ctypes.data if poly.size else None, poly.shape[0], xs.ctypes.data, y.ctypes.data,
                  nthreads)
    return y


def div_xplusc(poly: np.ndarray, c) -> np.ndarray:
    out = np.ascontiguousarray(poly, dtype=np.uint64).copy()
    cs = _scalar(c)
    lib().or_div_xplusc(out.ctypes.data if out.size else None, out.shape[0], cs.ctypes.data)
    return out


def naive_gp(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64)
    out = empty(a.shape[0])
    lib().or_naive_gp(a.ctypes.data, a.shape[0], out.ctypes.data)
    return out


def naive_div(a: np.ndarray, c):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    n = a.shape[0]
    q = empty(max(n - 1, 0))
    cs = _scalar(c)
    st = lib().or_naive_div(a.ctypes.data, n, cs.ctypes.data, q.ctypes.data if q.size else None)
    return q, st


def first_diff(a: np.ndarray, b: np.ndarray) -> int:
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, 4)
    b = np.ascontiguousarray(b, dtype=np.uint64).reshape(-1, 4)
    if a.shape != b.shape:
        return 0
    return int(lib().or_first_diff(a.ctypes.data, b.ctypes.data, a.shape[0]))


# ------------------------------------------------------ quotient constraints
# argument order of the reference's allmerge_kernel
# (PLONK/utils/zkp/cuda/zksnark_comute_gate_constraint.cu:6-19)
GATE_VECTORS = ["a_val", "b_val", "c_val", "d_val", "a_next_eval", "b_next_eval", "d_next_eval",
                "q_m", "q_l", "q_r", "q_o", "q_4", "q_c", "q_hl", "q_hr", "q_h4", "q_arith",
                "range", "logic", "fixed_group_add", "variable_group_add", "pi_eval_8n"]
GATE_SCALARS = ["four", "one", "two", "three", "kappa_range", "kappa_sq_range", "kappa_cu_range",
                "range_challenge", "P_D", "nine", "kappa_cu_logic", "eighteen", "eightyone",
                "eightythree", "kappa_qu_logic", "logic_challenge", "P_A", "kappa_fb", "kappa_sq_fb",
                "kappa_cu_fb", "fb_challenge", "kappa_vb", "kappa_sq_vb", "vb_challenge"]


def _vecs(xs):
    xs = [np.ascontiguousarray(x, dtype=np.uint64) for x in xs]
    return xs, (ctypes.c_void_p * len(xs))(*[x.ctypes.data for x in xs])


def quotient_identity(x, w, z, alpha, beta, gamma, ks) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.uint64)
    z = np.ascontiguousarray(z, dtype=np.uint64)
    n = x.shape[0]
    wk, wp = _vecs(w)
    kk, kp = _vecs([_scalar(k) for k in ks])
    al, be, ga = _scalar(alpha), _scalar(beta), _scalar(gamma)
    out = empty(n)
    lib().or_quotient_identity(x.ctypes.data, ctypes.cast(wp, ctypes.c_void_p), z.ctypes.data,
                               al.ctypes.data, be.ctypes.data, ga.ctypes.data,
                               ctypes.cast(kp, ctypes.c_void_p), out.ctypes.data, n)
    return out


def quotient_copy(sigma, mod, w, z_next, alpha, beta, gamma, result) -> np.ndarray:
    out = np.ascontiguousarray(result, dtype=np.uint64).copy()
    mod = np.ascontiguousarray(mod, dtype=np.uint64)
    z_next = np.ascontiguousarray(z_next, dtype=np.uint64)
    sk, sp = _vecs(sigma)
    wk, wp = _vecs(w)
    al, be, ga = _scalar(alpha), _scalar(beta), _scalar(gamma)
    lib().or_quotient_copy(ctypes.cast(sp, ctypes.c_void_p), mod.ctypes.data,
                           ctypes.cast(wp, ctypes.c_void_p), z_next.ctypes.data, al.ctypes.data,
                           be.ctypes.data, ga.ctypes.data, out.ctypes.data, out.shape[0])
    return out


def quotient_term_one(z, l1, one, result) -> np.ndarray:
    out = np.ascontiguousarray(result, dtype=np.uint64).copy()
    z = np.ascontiguousarray(z, dtype=np.uint64)
    l1 = np.ascontiguousarray(l1, dtype=np.uint64)
    o = _scalar(one)
    lib().or_quotient_term_one(z.ctypes.data, l1.ctypes.data, o.ctypes.data, out.ctypes.data,
                               out.shape[0])
    return out


def gate_constraint(vectors: dict, scalars: dict, sbox_alpha: int) -> np.ndarray:
    vk, vp = _vecs([vectors[k] for k in GATE_VECTORS])
    sk, sp = _vecs([_scalar(scalars[k]) for k in GATE_SCALARS])
    n = vk[0].shape[0]
    out = empty(n)
    lib().or_gate_constraint(ctypes.cast(vp, ctypes.c_void_p), ctypes.cast(sp, ctypes.c_void_p),
                             int(sbox_alpha), out.ctypes.data, n)
    return out


# ------------------------------------------------------------------------ G1
def g1_mul_gen(scalars, nthreads: int = 0) -> np.ndarray:
    """scalars (n, 4) -> affine points (n, 12): s_i * G."""
    s = np.ascontiguousarray(scalars, dtype=np.uint64).reshape(-1, 4)
    out = np.empty((s.shape[0], 12), dtype=np.uint64)
    lib().or_g1_mul_gen(s.ctypes.data, s.shape[0], out.ctypes.data, nthreads)
    return out


def g1_msm(points, scalars, nthreads: int = 0) -> np.ndarray:
    """sum_i scalars[i] * points[i] -> affine (12,)."""
    p = np.ascontiguousarray(points, dtype=np.uint64).reshape(-1, 12)
    s = np.ascontiguousarray(scalars, dtype=np.uint64).reshape(-1, 4)
    assert p.shape[0] == s.shape[0]
    out = np.empty(12, dtype=np.uint64)
    lib().or_g1_msm(p.ctypes.data if p.size else None, s.ctypes.data if s.size else None, p.shape[0],
                    out.ctypes.data, nthreads)
    return out


def g1_add(a, b) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(12)
    b = np.ascontiguousarray(b, dtype=np.uint64).reshape(12)
    out = np.empty(12, dtype=np.uint64)
    lib().or_g1_add(a.ctypes.data, b.ctypes.data, out.ctypes.data)
    return out
