"""NTT / INTT / LDE on the GPU through the C ABI, bit-exact against the oracle
at every size through 2^24, at the benchmark sizes (NTT/INTT 2^22, 2^24,
2^26; LDE 2^22 and 2^24 at lambda = 2, 3 in both coset forms), and through
size-independent properties at 2^25."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dev, host, table_elem

pytestmark = pytest.mark.gpu


def test_generator_matches_oracle(pp, O, cuda):
    for n, seed, first in ((1, 3, 0), (4096, 0x5EED, 0), (1000, 7, 123456)):
        assert (host(pp.random_fr(n, seed, first)) == O.random_fr(n, seed, first)).all()


@pytest.mark.parametrize("lg", list(range(0, 19)) + [20])
def test_ntt_bit_exact_all_sizes(pp, O, cuda, lg):
    """Every size through 2^18: one-block kernel to 2^8, two one-column-tile
    passes 2^9 .. 2^17, the tiled throughput plan from 2^18."""
    x = pp.random_fr(1 << lg, 100 + lg)
    xh = host(x)
    X = pp.ntt(x)
    want = O.ntt(xh)
    assert O.first_diff(host(X), want) == -1
    back = pp.intt(X)
    assert O.first_diff(host(back), xh) == -1
    assert O.first_diff(host(pp.intt(x)), O.ntt(xh, inverse=True)) == -1


def test_ntt_in_place_and_shipped_style_input(pp, O, cuda):
    lg = 14
    x = pp.random_fr(1 << lg, 9)
    want = O.ntt(host(x))
    pp.ntt(x, out=x)
    assert O.first_diff(host(x), want) == -1
    # low-entropy input like the reference's input.bin: zero, one, repeats
    a = np.zeros(((1 << lg), 4), np.uint64)
    a[1] = O.mont(1)
    a[2::7] = O.random_fr(1, 3)[0]
    assert O.first_diff(host(pp.ntt(dev(a))), O.ntt(a)) == -1


def test_ntt_of_delta_is_reference_root_table(pp, O, cuda, golden):
    """NTT(e_1)[k] = w^k: entry 1 must be forward_roots_of_unity[lg] of the
    reference's parameter header, entry 1 of the inverse its inverse root."""
    tables, _ = golden
    for lg in (5, 12, 20):
        e = np.zeros((1 << lg, 4), np.uint64)
        e[1] = O.mont(1)
        X = host(pp.ntt(dev(e)))
        assert (X[1] == table_elem(tables["forward_roots_of_unity"][lg])).all()
        Xi = host(pp.intt(dev(e)))
        # INTT(e_1)[1] = w^-1 / N
        want = O.fr_mul(table_elem(tables["inverse_roots_of_unity"][lg]),
                        table_elem(tables["domain_size_inverse"][lg]))
        assert (Xi[1] == want).all()


@pytest.mark.parametrize("lg", [19, 21, 22, 23, 24])
def test_ntt_full_size_bit_exact(pp, O, cuda, lg):
    """Every throughput-plan size through 2^24 with its shipped radix split
    (2^19: 10+9, 2^21: 6+6+9, 2^23: 9+6+8 ...) against the oracle."""
    x = pp.random_fr(1 << lg, 0x5EED0000 + lg)
    X = pp.ntt(x)
    assert O.first_diff(host(X), O.ntt(host(x))) == -1


@pytest.mark.parametrize("lg", [22, 24, 26])
def test_ntt_intt_benchmark_sizes_bit_exact(pp, O, cuda, lg):
    """The benchmark sizes, forward and inverse, every element against the
    oracle (which takes a few seconds per transform on 16 host cores)."""
    n = 1 << lg
    x = pp.random_fr(n, 0xA11CE + lg)
    xh = host(x)
    assert O.first_diff(host(pp.ntt(x)), O.ntt(xh)) == -1
    assert O.first_diff(host(pp.intt(x)), O.ntt(xh, inverse=True)) == -1


def test_ntt_2p25_properties(pp, O, cuda):
    """2^25: round trip and X[k] = p(w^k) at sampled k (first, last, random)."""
    import torch

    lg = 25
    n = 1 << lg
    x = pp.random_fr(n, 0xA11CE + lg)
    X = pp.ntt(x)
    assert torch.equal(pp.intt(X), x)
    xh, Xh = host(x), host(X)
    w = O.root_of_unity(lg)
    rng = np.random.default_rng(lg)
    for k in [0, 1, n - 1] + [int(v) for v in rng.integers(0, n, 2)]:
        pt = O.fr_pow(w, k)
        assert (O.evaluate(xh, pt) == Xh[k]).all(), k
    del X, Xh


@pytest.mark.parametrize("lg,lam", [(4, 1), (6, 2), (7, 2), (10, 2), (10, 3), (12, 3), (15, 2), (16, 2),
                                    (20, 2), (20, 3)])
def test_lde_modes_bit_exact(pp, O, cuda, lg, lam):
    x = pp.random_fr(1 << lg, 300 + lg + lam)
    xh = host(x)
    assert O.first_diff(host(pp.lde(x, lam, pp.LDE_COEFFS)), O.lde_coeffs(xh, lam)) == -1
    assert O.first_diff(host(pp.lde(x, lam, pp.LDE_EVALS)), O.lde_evals(xh, lam)) == -1
    assert O.first_diff(host(pp.lde(x, lam, pp.LDE_SPREAD)), O.lde_spread(xh, lam)) == -1


@pytest.mark.parametrize("lg,lam", [(22, 2), (22, 3), (24, 2), (24, 3)])
def test_lde_benchmark_sizes_bit_exact(pp, O, cuda, lg, lam):
    """The benchmark LDE sizes in all three forms, every one of the
    2^(lg+lam) outputs against the oracle: from coefficients (shift
    7^(2^lam)), from evaluations (INTT, then shift 7) and spread."""
    x = pp.random_fr(1 << lg, 0x1DE0 + 16 * lg + lam)
    xh = host(x)
    out = host(pp.lde(x, lam, pp.LDE_COEFFS))
    assert O.first_diff(out, O.lde_coeffs(xh, lam)) == -1
    del out
    out = host(pp.lde(x, lam, pp.LDE_EVALS))
    assert O.first_diff(out, O.lde_evals(xh, lam)) == -1
    del out
    # the spread form (the reference's naive_lde input layout): the oracle runs
    # the whole 2^(lg+lam)-point transform of the zero-spread input
    out = host(pp.lde(x, lam, pp.LDE_SPREAD))
    assert O.first_diff(out, O.lde_spread(xh, lam)) == -1
