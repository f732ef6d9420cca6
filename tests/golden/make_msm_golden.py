"""Golden vectors for the G1 multi-scalar multiplication, computed by the
reference's vendored blst (PLONK/blst, built unmodified from src/server.c and
src/assembly.S by `make -C oracle ref`).

Run where the reference sources are checked out; the output is committed:

    python tests/golden/make_msm_golden.py [/path/to/reference]

Writes ``msm.npz``:

* ``fq_P`` / ``fq_RR`` -- BLS12_381_P and BLS12_381_RR parsed as text from
  PLONK/utils/mont/cuda/ff/bls12-381.hpp;
* ``gen`` -- blst's generator (BLS12_381_G1, src/e1.c), affine Montgomery;
* per case ``<name>/points`` (n, 12), ``<name>/scalars`` (n, 4) and
  ``<name>/out`` (12,): blst_p1s_mult_pippenger of the points and scalars
  with nbits = 255, converted to affine (all zero = infinity).

Points are s * G for seeded scalars s (blst_p1_mult), plus edge cases: zero
and one scalars, r - 1, repeated points, P next to -P.  An all-zero input
point (infinity) is left out: blst's multi-point Pippenger reads it as a
coordinate pair rather than as infinity, so its result there is not a
reference behaviour; the GPU's handling of it is tested against the oracle.
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.join(HERE, "..", "..")
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

Q = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB
R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


def parse_fq(ref: str) -> dict:
    text = open(os.path.join(ref, "PLONK/utils/mont/cuda/ff/bls12-381.hpp")).read()
    out = {}
    for name in ("BLS12_381_P", "BLS12_381_RR"):
        m = re.search(r"\b" + name + r"\[12\]\s*=\s*\{(.*?)\};", text, re.S)
        assert m, name
        words = [int(w, 16) for w in re.findall(r"TO_CUDA_T\((0x[0-9a-fA-F]+)\)", m.group(1))]
        assert len(words) == 6, (name, words)
        out[name] = np.array(words, dtype=np.uint64)
    return out


def neg(point: np.ndarray) -> np.ndarray:
    p = point.copy()
    y = sum(int(p[6 + k]) << (64 * k) for k in range(6))
    y = (Q - y) % Q
    p[6:] = [(y >> (64 * k)) & (2**64 - 1) for k in range(6)]
    return p


def main(ref: str) -> None:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "REF=" + ref, "ref"], check=True)
    B = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libppblst.so"))
    sz = ctypes.c_size_t
    v = ctypes.c_void_p
    B.refg1_generator.argtypes = [v]
    B.refg1_mul_gen.argtypes = [v, sz, v]
    B.refg1_msm.argtypes = [v, v, sz, v]
    B.refg1_msm.restype = ctypes.c_int

    def mul_gen(s):
        s = np.ascontiguousarray(s, dtype=np.uint64)
        out = np.empty((s.shape[0], 12), np.uint64)
        B.refg1_mul_gen(s.ctypes.data, sz(s.shape[0]), out.ctypes.data)
        return out

    def msm(points, scalars):
        p = np.ascontiguousarray(points, dtype=np.uint64)
        s = np.ascontiguousarray(scalars, dtype=np.uint64)
        out = np.empty(12, np.uint64)
        assert B.refg1_msm(p.ctypes.data if p.size else None, s.ctypes.data if s.size else None,
                           sz(p.shape[0]), out.ctypes.data) == 0
        return out

    arrays = {}
    fq = parse_fq(ref)
    arrays["fq_P"] = fq["BLS12_381_P"]
    arrays["fq_RR"] = fq["BLS12_381_RR"]
    g = np.empty(12, np.uint64)
    B.refg1_generator(g.ctypes.data)
    arrays["gen"] = g

    seed = 0x5EED0E00
    cases = {}
    for n in (1, 2, 7, 64, 1000, 4099):
        seed += 1
        pts = mul_gen(O.random_fr(n, seed))
        sc = O.random_fr(n, seed + 1000)
        cases["rand_n%d" % n] = (pts, sc)
    # edge cases
    base = mul_gen(O.random_fr(16, 0xE1))
    sc = O.random_fr(16, 0xE2)
    sc[0] = 0
    sc[1] = [1, 0, 0, 0]
    rm1 = R - 1
    sc[2] = [(rm1 >> (64 * k)) & (2**64 - 1) for k in range(4)]
    pts = base.copy()
    pts[4] = pts[3]                      # repeated point
    pts[6] = neg(pts[5])                 # P and -P with equal scalars cancel
    sc[6] = sc[5]
    cases["edge_n16"] = (pts, sc)
    cases["cancel_n2"] = (np.stack([base[0], neg(base[0])]), np.stack([sc[3], sc[3]]))
    cases["small_scalars_n300"] = (mul_gen(O.random_fr(300, 0xE3)),
                                   np.array([[i % 7, 0, 0, 0] for i in range(300)], np.uint64))
    for name, (pts, sc) in cases.items():
        arrays[name + "/points"] = pts
        arrays[name + "/scalars"] = sc
        arrays[name + "/out"] = msm(pts, sc)
    np.savez_compressed(os.path.join(HERE, "msm.npz"), **arrays)
    print("wrote %d arrays" % len(arrays))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: %s <reference checkout>" % sys.argv[0])
    main(sys.argv[1])
