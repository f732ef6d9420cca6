"""The oracle's restatement of the PLONK quotient-constraint kernels against
golden vectors computed from the reference's own kernel expressions
(tests/golden/make_constraint_golden.py evaluates the right-hand sides of
zksnark_compute_permutation_constraint.cu:5-47 and
zksnark_comute_gate_constraint.cu:6-27 with Python integers mod r)."""
from __future__ import annotations

import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "constraints.npz")
GATE_CASES = ["gate_rand_a5_n64", "gate_small_a5_n33", "gate_rand_a2_n16", "gate_rand_a7_n16"]


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def perm_inputs(g, n):
    t = "perm_n%d/" % n
    get = lambda k: g[t + k]  # noqa: E731
    return t, get


@pytest.mark.parametrize("n", [1, 7, 64])
def test_permutation_terms_match_reference_expressions(O, gold, n):
    t, g = perm_inputs(gold, n)
    w = [g("w_l"), g("w_r"), g("w_o"), g("w_4")]
    sig = [g("left_sigma"), g("right_sigma"), g("out_sigma"), g("fourth_sigma")]
    ks = [g("k1")[0], g("k2")[0], g("k3")[0]]
    ident = O.quotient_identity(g("x"), w, g("z"), g("alpha")[0], g("beta")[0], g("gamma")[0], ks)
    assert np.array_equal(ident, g("identity"))
    cop = O.quotient_copy(sig, g("mod"), w, g("z_next"), g("alpha")[0], g("beta")[0], g("gamma")[0],
                          g("result"))
    assert np.array_equal(cop, g("copy"))
    one = O.quotient_term_one(g("z"), g("l1"), g("one")[0], g("result"))
    assert np.array_equal(one, g("term_one"))


@pytest.mark.parametrize("case", GATE_CASES)
def test_gate_constraint_matches_reference_expression(O, gold, case):
    t = case + "/"
    V = {k: gold[t + k] for k in O.GATE_VECTORS}
    S = {k: gold[t + k][0] for k in O.GATE_SCALARS}
    out = O.gate_constraint(V, S, int(gold[t + "SBOX_ALPHA"][0]))
    assert np.array_equal(out, gold[t + "out"])


def test_gate_oracle_is_sensitive_to_every_input(O, gold):
    """Each vector and scalar changes the output: no input is dropped."""
    t = "gate_rand_a5_n64/"
    V = {k: gold[t + k][:4].copy() for k in O.GATE_VECTORS}
    S = {k: gold[t + k][0].copy() for k in O.GATE_SCALARS}
    base = O.gate_constraint(V, S, 5)
    for k in O.GATE_VECTORS:
        V2 = dict(V)
        V2[k] = O.random_fr(4, 0xA11 + len(k))
        assert not np.array_equal(O.gate_constraint(V2, S, 5), base), k
    for k in O.GATE_SCALARS:
        S2 = dict(S)
        S2[k] = O.random_fr(1, 0xB22 + len(k))[0]
        assert not np.array_equal(O.gate_constraint(V, S2, 5), base), k
