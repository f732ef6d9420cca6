"""Golden vectors for the PLONK quotient-constraint operators, computed from
the reference's own kernel expressions.

Run where the reference sources are checked out (they do not travel with the
repository); the output is committed:

    python tests/golden/make_constraint_golden.py [/path/to/reference]

The right-hand sides of the reference's element-wise kernels are read as text:

* compute_quotient_identity_range_check_i, compute_quotient_copy_range_check_i
  and compute_quotient_term_check_one_i
  (PLONK/utils/zkp/cuda/zksnark_compute_permutation_constraint.cu:5-47);
* allmerge_kernel (PLONK/utils/zkp/cuda/zksnark_comute_gate_constraint.cu:6-30).

Each expression is parsed with Python's ``ast`` (C++ and Python agree on the
precedence of ``* + - ^`` and on left associativity) and evaluated over the
integers mod r.  ``x ^ p`` is the reference's mont_t power (mont_t.cuh:446-467).
The kernels compute on Montgomery forms; Montgomery multiplication is a ring
isomorphism, so evaluating the decoded values and re-encoding the result gives
the kernel's output exactly.

Writes ``constraints.npz``: for every case its inputs (vectors of n elements,
scalars of one element; 4 little-endian uint64 limbs, Montgomery form) and the
expected output.
"""
from __future__ import annotations

import ast
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", ".."))
from oracle import oracle as O  # noqa: E402

R_MOD = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
R_MONT = (1 << 256) % R_MOD
R_INV = pow(R_MONT, -1, R_MOD)

PERM_FILE = "PLONK/utils/zkp/cuda/zksnark_compute_permutation_constraint.cu"
GATE_FILE = "PLONK/utils/zkp/cuda/zksnark_comute_gate_constraint.cu"

GATE_VECTORS = ["a_val", "b_val", "c_val", "d_val", "a_next_eval", "b_next_eval", "d_next_eval",
                "q_m", "q_l", "q_r", "q_o", "q_4", "q_c", "q_hl", "q_hr", "q_h4", "q_arith",
                "range", "logic", "fixed_group_add", "variable_group_add", "pi_eval_8n"]
GATE_SCALARS = ["four", "one", "two", "three", "kappa_range", "kappa_sq_range", "kappa_cu_range",
                "range_challenge", "P_D", "nine", "kappa_cu_logic", "eighteen", "eightyone",
                "eightythree", "kappa_qu_logic", "logic_challenge", "P_A", "kappa_fb", "kappa_sq_fb",
                "kappa_cu_fb", "fb_challenge", "kappa_vb", "kappa_sq_vb", "vb_challenge"]


def kernel_exprs(path: str, lhs: str) -> list:
    """Right-hand sides of `lhs[tid] = ...;` in a kernel source, as Python text."""
    text = open(path).read()
    out = []
    for m in re.finditer(re.escape(lhs) + r"\[tid\]\s*=\s*(.*?);", text, re.S):
        e = m.group(1).replace("\\\n", " ")
        e = re.sub(r"\[tid\]|\[0\]", "", e)
        out.append(" ".join(e.split()))
    return out


def evaluate(expr: str, env: dict) -> int:
    def ev(node):
        if isinstance(node, ast.Name):
            return env[node.id]
        if isinstance(node, ast.Constant):
            return node.value
        if isinstance(node, ast.BinOp):
            a, b = ev(node.left), ev(node.right)
            if isinstance(node.op, ast.Add):
                return (a + b) % R_MOD
            if isinstance(node.op, ast.Sub):
                return (a - b) % R_MOD
            if isinstance(node.op, ast.Mult):
                return a * b % R_MOD
            if isinstance(node.op, ast.BitXor):  # mont_t operator^(int p), p >= 2
                assert isinstance(b, int) and b >= 2
                return pow(a, b, R_MOD)
        raise ValueError("unexpected node %s" % ast.dump(node))

    return ev(ast.parse(expr, mode="eval").body)


def dec(limbs) -> int:
    v = sum(int(x) << (64 * k) for k, x in enumerate(limbs))
    return v * R_INV % R_MOD


def enc(v: int) -> np.ndarray:
    m = v * R_MONT % R_MOD
    return np.array([(m >> (64 * k)) & (2**64 - 1) for k in range(4)], dtype=np.uint64)


def const_mont(v: int) -> np.ndarray:
    return enc(v % R_MOD)[None, :]


def main(ref: str) -> None:
    perm = kernel_exprs(os.path.join(ref, PERM_FILE), "result")
    assert len(perm) == 3, perm
    identity, copy, term_one = perm
    gate = kernel_exprs(os.path.join(ref, GATE_FILE), "gate_contributions")
    assert len(gate) == 1
    gate = gate[0]
    arrays = {}
    seed = 0x5EED0C00

    def vec(name, n):
        nonlocal seed
        seed += 1
        return O.random_fr(n, seed)

    # ---- permutation terms
    for n in (1, 7, 64):
        tag = "perm_n%d" % n
        names = ["x", "w_l", "w_r", "w_o", "w_4", "z", "z_next", "left_sigma", "right_sigma",
                 "out_sigma", "fourth_sigma", "mod", "l1", "result"]
        vals = {k: vec(k, n) for k in names}
        scal = {k: vec(k, 1) for k in ("alpha", "beta", "gamma", "k1", "k2", "k3", "one")}
        for k, a in list(vals.items()) + list(scal.items()):
            arrays[tag + "/" + k] = a
        ident = np.zeros((n, 4), np.uint64)
        cop = np.zeros((n, 4), np.uint64)
        one = np.zeros((n, 4), np.uint64)
        for i in range(n):
            env = {k: dec(v[i]) for k, v in vals.items()}
            env.update({k: dec(v[0]) for k, v in scal.items()})
            ident[i] = enc(evaluate(identity, env))
            cop[i] = enc(evaluate(copy, env))          # result + mod - ... (result = the input)
            one[i] = enc(evaluate(term_one, env))      # result + (z - one) * l1
        arrays[tag + "/identity"] = ident
        arrays[tag + "/copy"] = cop
        arrays[tag + "/term_one"] = one
    # ---- gate constraint: random scalars, then the natural small constants
    cases = [("gate_rand_a5_n64", 64, 5, False), ("gate_small_a5_n33", 33, 5, True),
             ("gate_rand_a2_n16", 16, 2, False), ("gate_rand_a7_n16", 16, 7, False)]
    small = {"one": 1, "two": 2, "three": 3, "four": 4, "nine": 9, "eighteen": 18,
             "eightyone": 81, "eightythree": 83}
    for tag, n, alpha, natural in cases:
        vals = {k: vec(k, n) for k in GATE_VECTORS}
        scal = {}
        for k in GATE_SCALARS:
            scal[k] = const_mont(small[k]) if (natural and k in small) else vec(k, 1)
        for k, a in list(vals.items()) + list(scal.items()):
            arrays[tag + "/" + k] = a
        arrays[tag + "/SBOX_ALPHA"] = np.array([alpha], dtype=np.int64)
        out = np.zeros((n, 4), np.uint64)
        for i in range(n):
            env = {k: dec(v[i]) for k, v in vals.items()}
            env.update({k: dec(v[0]) for k, v in scal.items()})
            env["SBOX_ALPHA"] = alpha
            out[i] = enc(evaluate(gate, env))
        arrays[tag + "/out"] = out
    np.savez_compressed(os.path.join(HERE, "constraints.npz"), **arrays)
    print("wrote %d arrays" % len(arrays))


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: %s <reference checkout>" % sys.argv[0])
    main(sys.argv[1])
