"""Element-wise Fr operators (pp_fr_binary / pp_fr_unary / pp_fr_pow /
pp_fr_powers / pp_fr_fill, the reference's add_mod ... repeat_to_poly) on the
GPU against the oracle, element by element, with the reference's edge
behaviour: the inverse of 0 is 0."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dev, host

pytestmark = pytest.mark.gpu

SIZES = [1, 7, 33, 4099]


def oracle_binary(O, op, a, b):
    f = {0: O.fr_add, 1: O.fr_sub, 2: O.fr_mul}
    out = np.empty_like(a)
    for i in range(a.shape[0]):
        y = b[0] if b.shape[0] == 1 else b[i]
        if op == 3:
            out[i] = O.fr_mul(a[i], O.fr_inv(y))  # fr_inv(0) = 0
        else:
            out[i] = f[op](a[i], y)
    return out


def with_zeros(x, idx):
    x = x.copy()
    for i in idx:
        if i < x.shape[0]:
            x[i] = 0
    return x


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("op", [0, 1, 2, 3])
def test_binary_elementwise_and_scalar(pp, O, cuda, n, op):
    P = pp.ppfr
    a = host(pp.random_fr(n, 0x900 + n))
    b = with_zeros(host(pp.random_fr(n, 0x910 + n)), [0, 5, 32, 4000])
    got = host(P.fr_binary(op, dev(a), dev(b)))
    assert O.first_diff(got, oracle_binary(O, op, a, b)) == -1
    if n > 1:
        s = host(pp.random_fr(1, 0x920 + n))
        got = host(P.fr_binary(op, dev(a), dev(s)))
        assert O.first_diff(got, oracle_binary(O, op, a, s)) == -1
        z = np.zeros((1, 4), np.uint64)  # division by a zero scalar gives 0
        got = host(P.fr_binary(op, dev(a), dev(z)))
        assert O.first_diff(got, oracle_binary(O, op, a, z)) == -1


@pytest.mark.parametrize("op", [0, 1, 2, 3])
def test_binary_in_place(pp, O, cuda, op):
    P = pp.ppfr
    n = 1000
    a = host(pp.random_fr(n, 0x930))
    b = with_zeros(host(pp.random_fr(n, 0x931)), [3, 999])
    want = oracle_binary(O, op, a, b)
    da, db = dev(a), dev(b)
    P.fr_binary(op, da, db, out=da)  # the reference's add_mod_(self, other) ...
    assert O.first_diff(host(da), want) == -1
    da, db = dev(a), dev(b)
    P.fr_binary(op, da, db, out=db)
    assert O.first_diff(host(db), want) == -1


@pytest.mark.parametrize("n", SIZES)
def test_unary(pp, O, cuda, n):
    P = pp.ppfr
    a = with_zeros(host(pp.random_fr(n, 0x940 + n)), [0, 31, 4098])
    neg = host(P.fr_unary(P.FR_NEG, dev(a)))
    inv = host(P.fr_unary(P.FR_INV, dev(a)))
    for i in range(n):
        assert (neg[i] == O.fr_neg(a[i])).all()
        assert (inv[i] == O.fr_inv(a[i])).all()
    d = dev(a)
    P.fr_unary(P.FR_INV, d, out=d)  # in place
    assert O.first_diff(host(d), inv) == -1


@pytest.mark.parametrize("e", [0, 1, 2, 3, 7, 65537, (1 << 64) - 1])
def test_pow(pp, O, cuda, e):
    P = pp.ppfr
    a = with_zeros(host(pp.random_fr(300, 0x950 + e % 1000)), [7])
    got = host(P.fr_pow(dev(a), e))
    for i in range(a.shape[0]):
        assert (got[i] == O.fr_pow(a[i], e)).all()


@pytest.mark.parametrize("n", [1, 2, 31, 32, 33, 1000, 5000])
def test_powers_and_fill(pp, O, cuda, n):
    P = pp.ppfr
    x = pp.random_fr(1, 0x960 + n)
    xh = host(x)[0]
    got = host(P.fr_powers(x, n))
    acc = O.mont(1)
    for i in range(n):
        assert (got[i] == acc).all(), i
        acc = O.fr_mul(acc, xh)
    fill = host(P.fr_fill(x, n))
    assert (fill == xh).all()


def test_large_division_round_trip(pp, cuda):
    """2^22 elements: (a / b) * b == a wherever b != 0, and 0 where b == 0."""
    P = pp.ppfr
    n = 1 << 22
    a, b = pp.random_fr(n, 0x970), pp.random_fr(n, 0x971)
    b[12345] = 0
    q = P.fr_binary(P.FR_DIV, a, b)
    back = P.fr_binary(P.FR_MUL, q, b)
    keep = cuda.ones(n, dtype=cuda.bool, device="cuda")
    keep[12345] = False
    assert cuda.equal(back[keep], a[keep])
    assert not q[12345].any()


def test_bad_arguments(pp, cuda):
    P = pp.ppfr
    a = pp.random_fr(8, 0x980)
    with pytest.raises(P.PPError):
        P.fr_binary(7, a, a)
    with pytest.raises(P.PPError):
        P.fr_unary(5, a)
    with pytest.raises(P.PPError):  # the scalar inside the output
        P.fr_binary(P.FR_ADD, a, a[2:3], out=a)
