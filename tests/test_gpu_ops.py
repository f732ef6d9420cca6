"""Grand product, permutation grand product, evaluation and division on the
GPU through the C ABI: bit-exact against the oracle and against the
reference's own CPU outputs (golden fixtures), including edge cases."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dev, host

pytestmark = pytest.mark.gpu

SIZES = [1, 2, 3, 4, 5, 31, 255, 256, 1000, 4096, 12345, 1 << 16, (1 << 20) + 7, 1 << 20]


@pytest.mark.parametrize("n", SIZES)
def test_gp_prefix(pp, O, cuda, n):
    x = pp.random_fr(n, 500 + n)
    want = O.gp_prefix(host(x))
    pp.gp_prefix_(x)
    assert O.first_diff(host(x), want) == -1


@pytest.mark.parametrize("n", [(1 << 22) + 3, 1 << 24])
def test_gp_prefix_large(pp, O, cuda, n):
    """The sizes that run 3 and 4 blocks per SM."""
    x = pp.random_fr(n, 550 + n % 1000)
    want = O.gp_prefix(host(x))
    pp.gp_prefix_(x)
    assert O.first_diff(host(x), want) == -1


@pytest.mark.parametrize("n", SIZES)
def test_eval(pp, O, cuda, n):
    p = pp.random_fr(n, 600 + n)
    z = pp.random_fr(1, 601 + n)
    y = pp.evaluate(p, z)
    assert (host(y)[0] == O.evaluate(host(p), host(z)[0])).all()


@pytest.mark.parametrize("n", SIZES)
def test_div(pp, O, cuda, n):
    p = pp.random_fr(n, 700 + n)
    c = pp.random_fr(1, 701 + n)
    want = O.div_xplusc(host(p), host(c)[0])
    pp.div_xplusc_(p, c)
    assert O.first_diff(host(p), want) == -1


# Chunk lengths K around the 16-coefficient groups of the evaluation's and the
# division's dot products (one group, one group and one term, two groups, ...):
# n = SMs x blocks per SM x 256 x K gives exactly K per thread (evaluation: 1
# block per SM up to 2^21 coefficients, 2 above; division: 2).
@pytest.mark.parametrize("k", [15, 16, 17, 31, 32, 33])
def test_eval_div_group_boundaries(pp, O, cuda, k):
    sms = cuda.cuda.get_device_properties(0).multi_processor_count
    for op, bps in (("eval", 1), ("div", 2)):
        n = sms * bps * 256 * k
        if op == "eval" and n > (1 << 21):
            n = sms * 2 * 256 * k
        p = pp.random_fr(n, 800 + k)
        c = pp.random_fr(1, 801 + k)
        if op == "eval":
            assert (host(pp.evaluate(p, c))[0] == O.evaluate(host(p), host(c)[0])).all(), (op, k, n)
        else:
            want = O.div_xplusc(host(p), host(c)[0])
            pp.div_xplusc_(p, c)
            assert O.first_diff(host(p), want) == -1, (op, k, n)


def test_reference_cpu_goldens(pp, O, cuda, golden):
    """GPU results vs the reference's naive_gp / naive_div outputs, using the
    conventions of its GPU operators (exclusive product; quotient of length n
    with a zero top entry)."""
    _, g = golden
    for name in g["case_names"]:
        name = str(name)
        x = dev(g[name + "_in"])
        pp.gp_prefix_(x)
        gx = host(x)
        assert (gx[1:] == g[name + "_naive_gp"][:-1]).all(), name
        assert (gx[0] == O.mont(1)).all()
        p = dev(g[name + "_in"])
        pp.div_xplusc_(p, dev(g[name + "_c"][None, :]))
        q = host(p)
        assert (q[:-1] == g[name + "_naive_div"]).all() and (q[-1] == 0).all(), name
    # evaluation at miss_ops.cu's own point on the shipped data
    x = g["inputbin12_in"]
    pt = g["eval_point_ref"]
    assert (host(pp.evaluate(dev(x), dev(pt[None, :])))[0] == O.evaluate(x, pt)).all()


def test_edge_values(pp, O, cuda):
    n = 1024
    a = np.zeros((n, 4), np.uint64)
    a[5] = O.mont(1)
    a[7] = O.from_int(O.R - 1)
    x = dev(a)
    pp.gp_prefix_(x)
    assert O.first_diff(host(x), O.gp_prefix(a)) == -1
    z0 = dev(np.zeros((1, 4), np.uint64))
    assert (host(pp.evaluate(dev(a), z0))[0] == a[0]).all()  # p(0) = c_0
    p = dev(a)
    pp.div_xplusc_(p, z0)  # division by X: shift down
    assert (host(p)[:-1] == a[1:]).all()
    empty = pp.ppfr.empty(0)
    y = pp.evaluate(empty, z0)
    assert (host(y) == 0).all()


@pytest.mark.parametrize("lg", [0, 1, 4, 10, 16, 20])
def test_gp_perm(pp, O, cuda, lg):
    n = 1 << lg
    w = [pp.random_fr(n, 800 + j) for j in range(3)]
    s = [pp.random_fr(n, 810 + j) for j in range(3)]
    beta, gamma = O.random_fr(1, 820)[0], O.random_fr(1, 821)[0]
    ks = [O.mont(1), O.mont(7), O.mont(13)]
    params = dev(np.stack([beta, gamma] + ks))
    z = pp.gp_perm(w, s, params)
    want = O.gp_perm([host(t) for t in w], [host(t) for t in s], beta, gamma, ks)
    assert O.first_diff(host(z), want) == -1


def test_gp_perm_zero_denominator(pp, O, cuda):
    """A zero denominator contributes the factor 0 (oracle: 0^-1 := 0)."""
    lg = 8
    n = 1 << lg
    w = [host(pp.random_fr(n, 900 + j)) for j in range(3)]
    s = [host(pp.random_fr(n, 910 + j)) for j in range(3)]
    beta, gamma = O.random_fr(1, 920)[0], O.random_fr(1, 921)[0]
    # make row 17's first denominator vanish: w0 + beta*s0 + gamma = 0
    s[0][17] = O.fr_mul(O.fr_neg(O.fr_add(w[0][17], gamma)), O.fr_inv(beta))
    ks = [O.mont(1), O.mont(7), O.mont(13)]
    z = pp.gp_perm([dev(t) for t in w], [dev(t) for t in s], dev(np.stack([beta, gamma] + ks)))
    want = O.gp_perm(w, s, beta, gamma, ks)
    zh = host(z)
    assert O.first_diff(zh, want) == -1
    assert (zh[18:] == 0).all() and not (zh[17] == 0).all()
