"""PLONK quotient-constraint operators on the GPU (pp_quotient_* and
pp_gate_constraint) against the reference-derived golden vectors and the
oracle, bit for bit."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import dev, host

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "constraints.npz")
GATE_CASES = ["gate_rand_a5_n64", "gate_small_a5_n33", "gate_rand_a2_n16", "gate_rand_a7_n16"]


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def perm_set(O, n, seed):
    names = ["x", "w_l", "w_r", "w_o", "w_4", "z", "z_next", "left_sigma", "right_sigma",
             "out_sigma", "fourth_sigma", "mod", "l1", "result"]
    vals = {k: O.random_fr(n, seed + i) for i, k in enumerate(names)}
    for i, k in enumerate(["alpha", "beta", "gamma", "k1", "k2", "k3", "one"]):
        vals[k] = O.random_fr(1, seed + 100 + i)
    return vals


def run_perm(P, vals):
    D = {k: dev(v) for k, v in vals.items()}
    w = [D["w_l"], D["w_r"], D["w_o"], D["w_4"]]
    sig = [D["left_sigma"], D["right_sigma"], D["out_sigma"], D["fourth_sigma"]]
    ks = [D["k1"], D["k2"], D["k3"]]
    ident = P.quotient_identity(D["x"], w, D["z"], D["alpha"], D["beta"], D["gamma"], ks)
    cop = D["result"].clone()
    P.quotient_copy_(cop, sig, D["mod"], w, D["z_next"], D["alpha"], D["beta"], D["gamma"])
    one = D["result"].clone()
    P.quotient_term_one_(one, D["z"], D["l1"], D["one"])
    fused = P.quotient_permutation(D["x"], w, D["z"], D["z_next"], sig, D["mod"], D["l1"],
                                   D["alpha"], D["beta"], D["gamma"], ks, D["one"])
    # the reference's three launches in sequence on one result buffer
    seq = P.quotient_identity(D["x"], w, D["z"], D["alpha"], D["beta"], D["gamma"], ks)
    P.quotient_copy_(seq, sig, D["mod"], w, D["z_next"], D["alpha"], D["beta"], D["gamma"])
    P.quotient_term_one_(seq, D["z"], D["l1"], D["one"])
    return host(ident), host(cop), host(one), host(fused), host(seq)


@pytest.mark.parametrize("n", [1, 7, 64])
def test_permutation_terms_match_golden(pp, cuda, gold, n):
    t = "perm_n%d/" % n
    vals = {k[len(t):]: v for k, v in gold.items() if k.startswith(t)}
    ident, cop, one, fused, seq = run_perm(pp.ppfr, vals)
    assert np.array_equal(ident, vals["identity"])
    assert np.array_equal(cop, vals["copy"])
    assert np.array_equal(one, vals["term_one"])
    assert np.array_equal(fused, seq)


@pytest.mark.parametrize("n", [255, 1000, (1 << 16) + 3])
def test_permutation_terms_match_oracle(pp, O, cuda, n):
    vals = perm_set(O, n, 0x9E0 + n)
    ident, cop, one, fused, seq = run_perm(pp.ppfr, vals)
    w = [vals["w_l"], vals["w_r"], vals["w_o"], vals["w_4"]]
    sig = [vals["left_sigma"], vals["right_sigma"], vals["out_sigma"], vals["fourth_sigma"]]
    ks = [vals["k1"][0], vals["k2"][0], vals["k3"][0]]
    a, b, g = vals["alpha"][0], vals["beta"][0], vals["gamma"][0]
    want_i = O.quotient_identity(vals["x"], w, vals["z"], a, b, g, ks)
    assert O.first_diff(ident, want_i) == -1
    assert O.first_diff(cop, O.quotient_copy(sig, vals["mod"], w, vals["z_next"], a, b, g,
                                             vals["result"])) == -1
    assert O.first_diff(one, O.quotient_term_one(vals["z"], vals["l1"], vals["one"][0],
                                                 vals["result"])) == -1
    want_f = O.quotient_term_one(vals["z"], vals["l1"], vals["one"][0],
                                 O.quotient_copy(sig, vals["mod"], w, vals["z_next"], a, b, g, want_i))
    assert O.first_diff(fused, want_f) == -1
    assert np.array_equal(fused, seq)


def gate_run(P, V, S, alpha):
    Vd = {k: dev(v) for k, v in V.items()}
    Sd = {k: dev(np.asarray(v).reshape(1, 4)) for k, v in S.items()}
    return host(P.gate_constraint(Vd, Sd, alpha))


@pytest.mark.parametrize("case", GATE_CASES)
def test_gate_matches_golden(pp, cuda, gold, case):
    P = pp.ppfr
    t = case + "/"
    V = {k: gold[t + k] for k in P.GATE_VECTORS}
    S = {k: gold[t + k][0] for k in P.GATE_SCALARS}
    out = gate_run(P, V, S, int(gold[t + "SBOX_ALPHA"][0]))
    assert np.array_equal(out, gold[t + "out"])


@pytest.mark.parametrize("n,alpha", [(1, 5), (777, 5), (4096, 3), ((1 << 15) + 1, 5)])
def test_gate_matches_oracle(pp, O, cuda, n, alpha):
    P = pp.ppfr
    V = {k: O.random_fr(n, 0x6A7E + i) for i, k in enumerate(P.GATE_VECTORS)}
    S = {k: O.random_fr(1, 0x5CA1 + i)[0] for i, k in enumerate(P.GATE_SCALARS)}
    out = gate_run(P, V, S, alpha)
    assert O.first_diff(out, O.gate_constraint(V, S, alpha)) == -1


SMALL = {"one": 1, "two": 2, "three": 3, "four": 4, "nine": 9, "eighteen": 18,
         "eightyone": 81, "eightythree": 83}


@pytest.mark.parametrize("n,off", [(1, None), (4097, None), ((1 << 15) + 3, None),
                                   (513, "one"), (513, "eightythree"), (513, "four")])
def test_gate_small_constants(pp, O, cuda, n, off):
    """The prover's natural constants (additions instead of multiplies) and
    the same with one of them off by one (the general form): both bit-exact."""
    P = pp.ppfr
    V = {k: O.random_fr(n, 0x7A7E + i) for i, k in enumerate(P.GATE_VECTORS)}
    S = {k: O.random_fr(1, 0x7CA1 + i)[0] for i, k in enumerate(P.GATE_SCALARS)}
    for k, v in SMALL.items():
        S[k] = O.mont(v + (k == off))
    out = gate_run(P, V, S, 5)
    assert O.first_diff(out, O.gate_constraint(V, S, 5)) == -1


def test_edge_cases_and_errors(pp, O, cuda):
    import torch
    P = pp.ppfr
    # n = 0 is a no-op
    e = P.empty(0)
    x = P.empty(1)
    assert P.quotient_identity(e, [e] * 4, e, x, x, x, [x] * 3, out=e).shape[0] == 0
    # S-box exponents below 2 are refused (the reference's power traps there)
    V = {k: P.random_fr(8, i) for i, k in enumerate(P.GATE_VECTORS)}
    S = {k: P.random_fr(1, 100 + i) for i, k in enumerate(P.GATE_SCALARS)}
    for bad in (0, 1, -5, 1 << 31):
        with pytest.raises(P.PPError) as err:
            P.gate_constraint(V, S, bad)
        assert err.value.status == 1
    # a missing input is refused before launch
    with pytest.raises(P.PPError) as err:
        P._perm_call("pp_quotient_copy", P._perm_args(z=V["a_val"]), P.empty(8), None)
    assert err.value.status == 1
    # zeros: every term vanishes when all vectors are zero and beta, gamma, one = 0
    n = 16
    zv = {k: np.zeros((n, 4), np.uint64) for k in P.GATE_VECTORS}
    zs = {k: np.zeros(4, np.uint64) for k in P.GATE_SCALARS}
    assert not gate_run(P, zv, zs, 5).any()
    torch.cuda.synchronize()
