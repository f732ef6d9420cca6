"""Bit-exact parity with outputs of the reference's own GPU operators.

``tests/golden/reference_gpu.npz`` was recorded on a GB300 by
``tests/golden/make_reference_gpu_golden.py``: the reference's sources, built
for sm_103a with its own flags, run on seeded inputs.  Large outputs are kept
as SHA-256 digests plus sampled elements, so each comparison below covers the
whole output, at the reference's own sizes:

* ``Ntt::forward`` / ``Intt::forward`` at 2^18 ... 2^26 -> ``pp_ntt`` (forward / inverse);
* ``our_ntt`` at 2^22, 2^24, 2^26 and ``standard4_ntt`` at 2^22, 2^24 (the
  same transform, host-resident) -> ``pp_ntt`` and ``pp_ntt_host``;
* ``our_lde`` at 2^20, 2^22, 2^24 with lambda = 2, 3 (N coefficients in, the
  coset extension p(7^(2^lambda) w^k) out) -> ``pp_lde`` mode 0;
* ``accumulate_mul_poly``, ``evaluate``, ``poly_div_poly`` at 2^10 ... 2^22
  -> ``pp_gp_prefix``, ``pp_eval``, ``pp_div_xplusc``.

Inputs are regenerated on the device by ``pp_random_fr`` from the stored
seeds (the generator equals the oracle's, which ``smoke()`` checks).
"""
from __future__ import annotations

import hashlib
import os

import numpy as np
import pytest

from conftest import ROOT, host

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_gpu.npz")


@pytest.fixture(scope="module")
def G():
    if not os.path.exists(GOLDEN):
        pytest.fail("tests/golden/reference_gpu.npz is missing")
    return dict(np.load(GOLDEN))


def _sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype=np.uint64).tobytes()).hexdigest()


def _check(G, key, out: np.ndarray):
    """out must equal the reference's output recorded under key."""
    if key + "_full" in G:
        want = G[key + "_full"]
        assert out.shape == want.shape
        bad = np.nonzero((out != want).any(axis=1))[0]
        assert bad.size == 0, f"{key}: first mismatch at {bad[:5]}"
        return
    idx = G[key + "_idx"]
    bad = np.nonzero((out[idx] != G[key + "_val"]).any(axis=1))[0]
    assert bad.size == 0, f"{key}: sampled elements differ at {idx[bad[:5]]}"
    assert _sha(out) == str(G[key + "_sha"]), f"{key}: SHA-256 of the output differs"


def _ntt_sizes(G):
    return sorted(int(k.split("_")[2]) for k in G if k.startswith("seed_ntt_"))


def test_golden_file_covers_the_reference_sizes(G):
    assert _ntt_sizes(G) == [18, 20, 22, 24, 26]
    for lg, lam in ((20, 2), (20, 3), (22, 2), (22, 3), (24, 2), (24, 3)):
        assert f"lde_{lg}_{lam}_sha" in G
    for lg in (22, 24, 26):
        assert f"ntt_split_{lg}_sha" in G


@pytest.mark.parametrize("lg", [18, 20, 22, 24, 26])
def test_ntt_and_intt_match_reference_gpu(pp, cuda, G, lg):
    x = pp.random_fr(1 << lg, int(G[f"seed_ntt_{lg}"]))
    fwd = host(pp.ntt(x))
    _check(G, f"ntt_fwd_{lg}", fwd)
    # the reference's --check-split / --check-baseline claim: our_ntt and
    # standard4_ntt equal Ntt::forward bit for bit
    for op in ("ntt_split", "ntt_std4"):
        if f"{op}_{lg}_sha" in G:
            assert _sha(fwd) == str(G[f"{op}_{lg}_sha"]), op
    del fwd
    _check(G, f"ntt_inv_{lg}", host(pp.intt(x)))


@pytest.mark.parametrize("lg", [22, 24])
def test_host_resident_ntt_matches_reference_our_ntt(pp, cuda, G, lg):
    x = pp.random_fr(1 << lg, int(G[f"seed_ntt_{lg}"]))
    xh = pp.ppfr.empty_pinned(1 << lg)
    xh.copy_(x.cpu())
    out = pp.ppfr.ntt_host(xh)
    cuda.cuda.synchronize()
    assert _sha(out.numpy().view(np.uint64).reshape(-1, 4)) == str(G[f"ntt_split_{lg}_sha"])


@pytest.mark.parametrize("lg,lam", [(20, 2), (20, 3), (22, 2), (22, 3), (24, 2), (24, 3)])
def test_lde_matches_reference_our_lde(pp, cuda, G, lg, lam):
    x = pp.random_fr(1 << lg, int(G[f"seed_lde_{lg}_{lam}"]))
    out = pp.lde(x, lam, pp.LDE_COEFFS)
    del x
    _check(G, f"lde_{lg}_{lam}", host(out))


@pytest.mark.parametrize("lg", [10, 16, 20, 22])
def test_scans_match_reference_gpu(pp, cuda, G, lg):
    s, sx, sc = (int(v) for v in G[f"seed_ops_{lg}"])
    n = 1 << lg
    a = pp.random_fr(n, s)
    x = pp.random_fr(1, sx)
    c = pp.random_fr(1, sc)
    g = a.clone()
    pp.gp_prefix_(g)
    _check(G, f"gp_{lg}", host(g))
    y = host(pp.evaluate(a, x))
    assert (y == G[f"eval_{lg}_full"]).all(), "evaluation differs"
    d = a.clone()
    pp.div_xplusc_(d, c)
    _check(G, f"div_{lg}", host(d))
