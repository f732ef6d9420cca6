"""G1 multi-scalar multiplication on the GPU (pp_msm_g1) against golden
vectors from the reference's vendored blst and against the oracle, bit for bit
on the affine result."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

GOLD = os.path.join(ROOT, "tests", "golden", "msm.npz")
CASES = ["rand_n1", "rand_n2", "rand_n7", "rand_n64", "rand_n1000", "rand_n4099", "edge_n16",
         "cancel_n2", "small_scalars_n300"]


def dev(a, torch):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def affine(out):
    """(3, 6) Jacobian with Z = 1 (or all zero) -> (12,) affine uint64."""
    o = out.cpu().numpy().view(np.uint64)
    if not o[2].any():
        assert not o.any()
        return np.zeros(12, np.uint64)
    return np.concatenate([o[0], o[1]])


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


@pytest.mark.parametrize("case", CASES)
def test_msm_matches_blst(pp, cuda, gold, case):
    out = pp.ppfr.msm_g1(dev(gold[case + "/points"], cuda), dev(gold[case + "/scalars"], cuda))
    assert np.array_equal(affine(out), gold[case + "/out"])


@pytest.mark.parametrize("n", [3, 100, 5000, 70000])
def test_msm_matches_oracle(pp, O, cuda, n):
    pts = O.g1_mul_gen(O.random_fr(n, 0xAB0 + n))
    sc = O.random_fr(n, 0xAC0 + n)
    out = pp.ppfr.msm_g1(dev(pts, cuda), dev(sc, cuda))
    assert np.array_equal(affine(out), O.g1_msm(pts, sc))


def test_msm_edge_cases(pp, O, cuda):
    P = pp.ppfr
    pts = O.g1_mul_gen(O.random_fr(64, 0xAD0))
    sc = O.random_fr(64, 0xAD1)
    # infinity inputs contribute nothing
    p2 = pts.copy()
    p2[5] = 0
    p2[40] = 0
    assert np.array_equal(affine(P.msm_g1(dev(p2, cuda), dev(sc, cuda))), O.g1_msm(p2, sc))
    # full 256-bit scalars (top bit set): exact, as the windows cover 257 bits
    big = sc.copy()
    big[:, 3] |= np.uint64(1 << 63)
    assert np.array_equal(affine(P.msm_g1(dev(pts, cuda), dev(big, cuda))), O.g1_msm(pts, big))
    # all-zero scalars and n = 0 give infinity
    z = np.zeros_like(sc)
    assert not affine(P.msm_g1(dev(pts, cuda), dev(z, cuda))).any()
    e = cuda.empty((0, 12), dtype=cuda.int64, device="cuda")
    assert not affine(P.msm_g1(e, cuda.empty((0, 4), dtype=cuda.int64, device="cuda"))).any()
    # every point in one bucket of every window: identical scalars
    same = np.repeat(sc[:1], 64, axis=0)
    assert np.array_equal(affine(P.msm_g1(dev(pts, cuda), dev(same, cuda))), O.g1_msm(pts, same))


def test_msm_large_equal_scalars(pp, O, cuda):
    """Buckets far larger than one thread's group (all scalars equal over
    40 000 points): the multi-level bucket sums."""
    P = pp.ppfr
    base = O.g1_mul_gen(O.random_fr(500, 0xAF0))
    n = 40000
    pts = np.ascontiguousarray(np.tile(base, (n // 500, 1)))
    sc = np.repeat(O.random_fr(1, 0xAF1), n, axis=0)
    # sum = s * (n / 500) * sum(base)
    want = O.g1_msm(pts, sc)
    assert np.array_equal(affine(P.msm_g1(dev(pts, cuda), dev(sc, cuda))), want)


def test_msm_repeatable(pp, O, cuda):
    P = pp.ppfr
    pts = O.g1_mul_gen(O.random_fr(3000, 0xAE0))
    sc = O.random_fr(3000, 0xAE1)
    a = affine(P.msm_g1(dev(pts, cuda), dev(sc, cuda)))
    b = affine(P.msm_g1(dev(pts, cuda), dev(sc, cuda)))
    assert np.array_equal(a, b)


# ---- fixed-base form (pp_msm_g1_bases_create / pp_msm_g1_fixed)
@pytest.mark.parametrize("case", CASES)
def test_fixed_msm_matches_blst(pp, cuda, gold, case):
    bases = pp.ppfr.MsmBases(dev(gold[case + "/points"], cuda))
    out = bases.msm(dev(gold[case + "/scalars"], cuda))
    assert np.array_equal(affine(out), gold[case + "/out"])


@pytest.mark.parametrize("n,c", [(1, 0), (2, 0), (100, 0), (3000, 0), (500, 6), (500, 13), (700, 20),
                                 (70000, 0)])
def test_fixed_msm_matches_plain_and_oracle(pp, O, cuda, n, c):
    P = pp.ppfr
    pts = O.g1_mul_gen(O.random_fr(n, 0xB10 + n))
    sc = O.random_fr(n, 0xB20 + n)
    bases = P.MsmBases(dev(pts, cuda), window_bits=c)
    if c:
        assert bases.window_bits == c
    assert bases.table_bytes == (256 // bases.window_bits + 1) * n * 96
    got = affine(bases.msm(dev(sc, cuda)))
    assert np.array_equal(got, affine(P.msm_g1(dev(pts, cuda), dev(sc, cuda))))
    if n <= 5000:
        assert np.array_equal(got, O.g1_msm(pts, sc))
    # the same tables serve another scalar vector
    sc2 = O.random_fr(n, 0xB30 + n)
    assert np.array_equal(affine(bases.msm(dev(sc2, cuda))),
                          affine(P.msm_g1(dev(pts, cuda), dev(sc2, cuda))))
    bases.close()


def test_fixed_msm_edge_cases(pp, O, cuda):
    P = pp.ppfr
    n = 64
    pts = O.g1_mul_gen(O.random_fr(n, 0xB40))
    pts[7] = 0  # infinity inputs: their tables are infinity
    pts[33] = 0
    sc = O.random_fr(n, 0xB41)
    bases = P.MsmBases(dev(pts, cuda), window_bits=8)
    assert np.array_equal(affine(bases.msm(dev(sc, cuda))), O.g1_msm(pts, sc))
    big = sc.copy()
    big[:, 3] |= np.uint64(1 << 63)
    big[3] = np.uint64(0xFFFFFFFFFFFFFFFF)  # 2^256 - 1
    assert np.array_equal(affine(bases.msm(dev(big, cuda))), O.g1_msm(pts, big))
    assert not affine(bases.msm(dev(np.zeros_like(sc), cuda))).any()
    # every window digit of every scalar is 37: all W n entries share one bucket
    s = sum(37 << (8 * w) for w in range(32))
    same = np.array([[(s >> (64 * k)) & 0xFFFFFFFFFFFFFFFF for k in range(4)]] * n, dtype=np.uint64)
    assert np.array_equal(affine(bases.msm(dev(same, cuda))), O.g1_msm(pts, same))
    # repeated points
    rep = np.ascontiguousarray(np.tile(pts[:8], (8, 1)))
    b2 = P.MsmBases(dev(rep, cuda))
    assert np.array_equal(affine(b2.msm(dev(sc, cuda))), O.g1_msm(rep, sc))


def test_fixed_msm_bad_arguments(pp, cuda):
    P = pp.ppfr
    pts = cuda.zeros((4, 12), dtype=cuda.int64, device="cuda")
    with pytest.raises(P.PPError):
        P.MsmBases(pts, window_bits=5)
    with pytest.raises(P.PPError):
        P.MsmBases(pts, window_bits=21)
    with pytest.raises(P.PPError):
        P.MsmBases(cuda.zeros((0, 12), dtype=cuda.int64, device="cuda"))


def test_g1_mul_gen_matches_oracle_and_blst(pp, O, cuda, gold):
    """pp_g1_mul_gen: s G for plain 256-bit scalars, including 1 (blst's
    generator itself), 0 and the group order r (infinity), and 2^256 - 1."""
    P = pp.ppfr
    r = [0xFFFFFFFF00000001, 0x53BDA402FFFE5BFE, 0x3339D80809A1D805, 0x73EDA753299D7D48]
    extra = np.array([[1, 0, 0, 0], [0, 0, 0, 0], r, [0xFFFFFFFFFFFFFFFF] * 4], dtype=np.uint64)
    sc = np.concatenate([O.random_fr(300, 0xB50), extra])
    got = P.g1_mul_gen(dev(sc, cuda)).cpu().numpy().view(np.uint64)
    assert np.array_equal(got, O.g1_mul_gen(sc))
    assert np.array_equal(got[300], gold["gen"])
    assert not got[301].any() and not got[302].any()
