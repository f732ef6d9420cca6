"""Generate the golden fixtures in this directory from the reference itself.

Run where the reference sources are checked out (they do not travel with the
repository); the outputs are committed so that every other machine can check
against them:

    python tests/golden/make_golden.py [/path/to/reference]

What it writes (all Fr values: 4 little-endian uint64 limbs, Montgomery form):

* ``ntt_tables.json`` -- the reference's NTT constant tables, parsed as text
  from PLONK/utils/zkp/cuda/zksnark_ntt/parameters/bls12_381.h:8-183
  (group_gen, group_gen_inverse, forward/inverse roots of unity for every
  2^k, k <= 32, and the 2^-k domain-size inverses).
* ``reference_cpu.npz`` -- outputs of the reference's own CPU code, compiled
  from its sources by oracle/Makefile (target ``ref``):
    - blst field products, sums, differences and inverses of seeded pairs
      (cpu::BLS12_381_Fr_G1, PLONK/utils/mont/cpu/ff/bls12-381.hpp);
    - ``naive_gp`` (miss_ops.cu:34-47) and ``naive_div`` (miss_ops.cu:49-87)
      on seeded inputs of 2^1, 2^4, 2^10 and 2^12 elements, and on the first
      2^12 elements of the reference's shipped ``input.bin`` with the eval
      point and divisor constants hard-coded in miss_ops.cu:133-135,163-165.
"""
from __future__ import annotations

import json
import os
import re
import sys
import zipfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import oracle as O  # noqa: E402

SEED_BASE = 0x5EED0000


def parse_tables(ref: str) -> dict:
    path = os.path.join(ref, "PLONK/utils/zkp/cuda/zksnark_ntt/parameters/bls12_381.h")
    text = open(path).read()
    # only the BLS12_381_Fr_G1 specialisation is in this header
    out = {}
    for name in ("group_gen", "group_gen_inverse", "forward_roots_of_unity",
                 "inverse_roots_of_unity", "domain_size_inverse"):
        m = re.search(r"\b" + name + r"\s*=\s*\{([^}]*)\}", text)
        assert m, name
        words = [int(w, 16) for w in re.findall(r"0x[0-9a-fA-F]+", m.group(1))]
        assert len(words) % 8 == 0
        elems = []
        for e in range(len(words) // 8):
            limbs = [words[8 * e + 2 * k] | (words[8 * e + 2 * k + 1] << 32) for k in range(4)]
            elems.append(["%016x" % v for v in limbs])
        out[name] = elems
    return out


def read_input_bin(ref: str, n: int) -> np.ndarray:
    with zipfile.ZipFile(os.path.join(ref, "input.bin.zip")) as z:
        with z.open("input.bin") as f:
            raw = f.read(n * 32)
    return np.frombuffer(raw, dtype=np.uint64).reshape(n, 4).copy()


def main(ref: str) -> None:
    O.build(ref=True)
    R = O.ref_lib()
    assert R is not None, "reference harness did not build"
    tables = parse_tables(ref)
    with open(os.path.join(HERE, "ntt_tables.json"), "w") as f:
        json.dump(tables, f, indent=0)

    arrays = {}
    n = 256
    a = O.random_fr(n, SEED_BASE + 1)
    b = O.random_fr(n, SEED_BASE + 2)
    b[0] = 0  # edge values: zero, one, r-1
    b[1] = O.from_int(O.ONE_MONT)
    a[2] = O.from_int(O.R - 1)
    arrays["field_a"], arrays["field_b"] = a, b
    for op in ("mul", "add", "sub"):
        out = O.empty(n)
        getattr(R, "ref_fr_" + op)(a.ctypes.data, b.ctypes.data, out.ctypes.data, n)
        arrays["field_" + op] = out
    inv = O.empty(n)
    R.ref_fr_inv(a.ctypes.data, inv.ctypes.data, n)
    arrays["field_inv_a"] = inv

    cases = []
    for lg in (1, 4, 10, 12):
        cases.append(("seed%d" % lg, lg, O.random_fr(1 << lg, SEED_BASE + 100 + lg),
                      O.random_fr(1, SEED_BASE + 200 + lg)[0]))
    # shipped data with miss_ops.cu's own constants
    c_ref = np.array([123456789123456789, 987654321987654321, 1122334455667788, 1122334455667788],
                     dtype=np.uint64)
    cases.append(("inputbin12", 12, read_input_bin(ref, 1 << 12), c_ref))
    arrays["eval_point_ref"] = np.array([123456789, 987654321, 1122334455, 6677889900], dtype=np.uint64)
    names = []
    for name, lg, x, c in cases:
        g = O.empty(1 << lg)
        R.ref_naive_gp(lg, x.ctypes.data, g.ctypes.data)
        q = O.empty((1 << lg) - 1)
        R.ref_naive_div(lg, x.ctypes.data, c.ctypes.data, q.ctypes.data)
        arrays[name + "_in"] = x
        arrays[name + "_c"] = c
        arrays[name + "_naive_gp"] = g
        arrays[name + "_naive_div"] = q
        names.append(name)
    arrays["case_names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "reference_cpu.npz"), **arrays)
    print("wrote", sorted(arrays))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: %s <reference checkout>" % sys.argv[0])
    main(sys.argv[1])
