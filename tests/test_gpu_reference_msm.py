"""pp_msm_g1 against the reference's own GPU multi-scalar multiplication,
``multi_scalar_mult`` (PLONK/utils/function.cu:396-412), bit for bit on the
affine result.

``tests/golden/reference_gpu_msm.npz`` was recorded on a GB300 by
``tests/golden/make_reference_msm_golden.py`` (the reference's sources built
for sm_103a with its own flags).  It keeps the seeds of each input and the
reference's result as it returns it: Jacobian X, Y, Z over Fq in Montgomery
form.  The points are regenerated by the oracle's g1_mul_gen, the scalars by
its random_fr."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

from conftest import ROOT, dev

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_gpu_msm.npz")
Q = 0x1A0111EA397FE69A4B1BA7B6434BACD764774B84F38512BF6730D2A0F6B0F6241EABFFFEB153FFFFB9FEFFFFFFFFAAAB
R_MONT = pow(2, 384, Q)
R_INV = pow(R_MONT, -1, Q)

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from make_reference_msm_golden import SIZES, inputs, seeds_for  # noqa: E402


def fq_int(words) -> int:
    return sum(int(w) << (64 * i) for i, w in enumerate(words))


def fq_words(x: int) -> np.ndarray:
    return np.array([(x >> (64 * i)) & (2**64 - 1) for i in range(6)], dtype=np.uint64)


def jacobian_to_affine(jac: np.ndarray) -> np.ndarray:
    """Jacobian (X, Y, Z), Montgomery -> affine (x, y), Montgomery, 12 words
    (all zero for infinity)."""
    X, Y, Z = (fq_int(jac[6 * k:6 * k + 6]) * R_INV % Q for k in range(3))
    if Z == 0:
        return np.zeros(12, np.uint64)
    zi = pow(Z, -1, Q)
    x = X * zi * zi % Q
    y = Y * zi * zi * zi % Q
    return np.concatenate([fq_words(x * R_MONT % Q), fq_words(y * R_MONT % Q)])


@pytest.fixture(scope="module")
def G():
    if not os.path.exists(GOLDEN):
        pytest.fail("tests/golden/reference_gpu_msm.npz is missing")
    return dict(np.load(GOLDEN))


@pytest.mark.parametrize("lg", SIZES)
def test_msm_matches_reference_gpu(pp, cuda, G, lg):
    points, scalars = inputs(lg)
    assert [int(v) for v in G[f"msm_{lg}_seeds"]] == list(seeds_for(lg))
    want = jacobian_to_affine(G[f"msm_{lg}_jacobian"])
    out = pp.ppfr.msm_g1(dev(points), dev(scalars)).cpu().numpy().view(np.uint64)
    got = np.zeros(12, np.uint64) if not out[2].any() else np.concatenate([out[0], out[1]])
    assert (got == want).all()
