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
