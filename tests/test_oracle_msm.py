"""The oracle's G1 multi-scalar multiplication against golden vectors made by
the reference's vendored blst (tests/golden/make_msm_golden.py), and the
field constants against the reference's BLS12_381_P / BLS12_381_RR."""
from __future__ import annotations

import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "msm.npz")
Q = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def to_int(limbs):
    return sum(int(w) << (64 * k) for k, w in enumerate(limbs))


def test_field_constants_match_reference(gold):
    assert to_int(gold["fq_P"]) == Q
    assert to_int(gold["fq_RR"]) == pow(2, 768, Q)


def test_generator_is_blst_generator(O, gold):
    one = np.array([1, 0, 0, 0], np.uint64)
    assert np.array_equal(O.g1_mul_gen(one)[0], gold["gen"])
    # on the curve y^2 = x^3 + 4 (decoded from Montgomery form)
    rinv = pow(2**384, -1, Q)
    x, y = to_int(gold["gen"][:6]) * rinv % Q, to_int(gold["gen"][6:]) * rinv % Q
    assert (y * y - x ** 3 - 4) % Q == 0


@pytest.mark.parametrize("case", ["rand_n1", "rand_n2", "rand_n7", "rand_n64", "rand_n1000",
                                  "rand_n4099", "edge_n16", "cancel_n2", "small_scalars_n300"])
def test_msm_matches_blst(O, gold, case):
    got = O.g1_msm(gold[case + "/points"], gold[case + "/scalars"])
    assert np.array_equal(got, gold[case + "/out"])


def test_infinity_inputs_contribute_nothing(O, gold):
    p = gold["rand_n7/points"].copy()
    s = gold["rand_n7/scalars"]
    base = O.g1_msm(p[1:], s[1:])
    p[0] = 0
    assert np.array_equal(O.g1_msm(p, s), base)
    assert not O.g1_msm(p[:0], s[:0]).any()
