"""The oracle, pinned against the reference: its NTT constant tables, its blst
field (reference_cpu.npz) and its own CPU operators naive_gp / naive_div; plus
big-integer restatements for the operators the reference has no CPU code for."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import table_elem

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001


def test_root_tables_match_reference(O, golden):
    tables, _ = golden
    assert (table_elem(tables["group_gen"][0]) == O.mont(7)).all()
    assert (table_elem(tables["group_gen_inverse"][0]) == O.fr_inv(O.mont(7))).all()
    for k in range(33):
        assert (table_elem(tables["forward_roots_of_unity"][k]) == O.root_of_unity(k)).all(), k
        assert (table_elem(tables["inverse_roots_of_unity"][k]) == O.root_of_unity(k, True)).all(), k
        assert (table_elem(tables["domain_size_inverse"][k]) == O.fr_inv(O.mont(1 << k))).all(), k


def test_field_ops_match_reference_blst(O, golden):
    _, g = golden
    a, b = g["field_a"], g["field_b"]
    for i in range(a.shape[0]):
        assert (O.fr_mul(a[i], b[i]) == g["field_mul"][i]).all()
        assert (O.fr_add(a[i], b[i]) == g["field_add"][i]).all()
        assert (O.fr_sub(a[i], b[i]) == g["field_sub"][i]).all()
        assert (O.fr_inv(a[i]) == g["field_inv_a"][i]).all()
        x, y = O.unmont(a[i]), O.unmont(b[i])
        assert O.unmont(g["field_mul"][i]) == x * y % R


def test_reference_cpu_operators(O, golden):
    """naive_gp / naive_div restated == the reference's own output; the GPU-side
    conventions (exclusive product, length-n quotient) follow from them."""
    _, g = golden
    for name in g["case_names"]:
        name = str(name)
        x, c = g[name + "_in"], g[name + "_c"]
        assert (O.naive_gp(x) == g[name + "_naive_gp"]).all(), name
        q, st = O.naive_div(x, c)
        assert st == 0 and (q == g[name + "_naive_div"]).all(), name
        ex = O.gp_prefix(x)
        assert (ex[1:] == g[name + "_naive_gp"][:-1]).all(), name
        assert (ex[0] == O.mont(1)).all()
        d = O.div_xplusc(x, c)
        assert (d[:-1] == g[name + "_naive_div"]).all() and (d[-1] == 0).all(), name


def test_oracle_against_live_reference(O):
    """Where the reference sources are present, its compiled CPU code agrees on fresh inputs."""
    ref = O.ref_lib()
    if ref is None:
        pytest.skip("reference sources not present on this machine")
    for lg in (3, 9):
        x = O.random_fr(1 << lg, 77 + lg)
        g = O.empty(1 << lg)
        ref.ref_naive_gp(lg, x.ctypes.data, g.ctypes.data)
        assert (g == O.naive_gp(x)).all()
        c = O.random_fr(1, 99)[0]
        q = O.empty((1 << lg) - 1)
        ref.ref_naive_div(lg, x.ctypes.data, c.ctypes.data, q.ctypes.data)
        assert (q == O.naive_div(x, c)[0]).all()


def _ints(a):
    return [O_unmont(r) for r in a]


def O_unmont(row):
    x = int(row[0]) | (int(row[1]) << 64) | (int(row[2]) << 128) | (int(row[3]) << 192)
    return x * pow(1 << 256, -1, R) % R


@pytest.mark.parametrize("lg", [0, 1, 2, 3, 5])
def test_ntt_is_the_dft(O, lg):
    n = 1 << lg
    x = O.random_fr(n, 1000 + lg)
    X = O.ntt(x)
    w = O_unmont(O.root_of_unity(lg))
    xi = [O_unmont(r) for r in x]
    for k in range(n):
        assert O_unmont(X[k]) == sum(xi[j] * pow(w, j * k, R) for j in range(n)) % R
    assert (O.ntt(X, inverse=True) == x).all()


@pytest.mark.parametrize("lg,lam", [(2, 1), (3, 2), (4, 3)])
def test_lde_forms(O, lg, lam):
    n, m = 1 << lg, 1 << (lg + lam)
    a = O.random_fr(n, 2000 + lg)
    ai = [O_unmont(r) for r in a]
    wL = O_unmont(O.root_of_unity(lg + lam))
    # reference form: coefficients in, shift 7^(2^lam)
    h = pow(7, 1 << lam, R)
    out = O.lde_coeffs(a, lam)
    for k in range(m):
        pt = h * pow(wL, k, R) % R
        assert O_unmont(out[k]) == sum(ai[i] * pow(pt, i, R) for i in range(n)) % R
    # evaluations in, shift 7
    coeffs = [O_unmont(r) for r in O.ntt(a, inverse=True)]
    out = O.lde_evals(a, lam)
    for k in range(m):
        pt = 7 * pow(wL, k, R) % R
        assert O_unmont(out[k]) == sum(coeffs[i] * pow(pt, i, R) for i in range(n)) % R
    # naive_lde spread: equals the N-point NTT at k mod N
    out = O.lde_spread(a, lam)
    X = O.ntt(a)
    for k in range(m):
        assert (out[k] == X[k % n]).all()


def test_eval_and_div_bigint(O):
    n = 257
    p = O.random_fr(n, 31)
    x = O.random_fr(1, 32)[0]
    pi = [O_unmont(r) for r in p]
    xi = O_unmont(x)
    assert O_unmont(O.evaluate(p, x)) == sum(pi[i] * pow(xi, i, R) for i in range(n)) % R
    assert (O.evaluate(O.empty(0), x) == 0).all()
    q = [O_unmont(r) for r in O.div_xplusc(p, x)]
    # p(X) = (X + c) q(X) + p(-c)
    z = (-xi) % R
    rem = sum(pi[i] * pow(z, i, R) for i in range(n)) % R
    assert q[-1] == 0
    for i in range(n):
        lhs = pi[i]
        rhs = ((q[i - 1] if i >= 1 else 0) + xi * q[i] + (rem if i == 0 else 0)) % R
        assert lhs == rhs, i


def test_gp_perm_bigint(O):
    lg = 4
    n = 1 << lg
    w = [O.random_fr(n, 40 + j) for j in range(3)]
    s = [O.random_fr(n, 50 + j) for j in range(3)]
    beta, gamma = O.random_fr(1, 60)[0], O.random_fr(1, 61)[0]
    ks = [O.mont(1), O.mont(7), O.mont(13)]
    z = O.gp_perm(w, s, beta, gamma, ks)
    om = O_unmont(O.root_of_unity(lg))
    b, g = O_unmont(beta), O_unmont(gamma)
    kk = [1, 7, 13]
    acc = 1
    for i in range(n):
        assert O_unmont(z[i]) == acc, i
        num = den = 1
        for j in range(3):
            wj = O_unmont(w[j][i])
            num = num * (wj + b * kk[j] * pow(om, i, R) + g) % R
            den = den * (wj + b * O_unmont(s[j][i]) + g) % R
        acc = acc * num * pow(den, -1, R) % R


def test_random_generator_is_canonical_and_seeded(O):
    a = O.random_fr(4096, 5)
    assert all(O.to_int(r) < R for r in a)
    assert (O.random_fr(4096, 5) == a).all()
    assert (O.random_fr(96, 5, first_index=4000) == a[4000:]).all()
    assert not (O.random_fr(4096, 6) == a).all()
