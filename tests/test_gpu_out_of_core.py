"""The out-of-core transform (pp_ntt_out_of_core): input, output and the
intermediate buffer stay in page-locked host memory, every pass reads and
writes host memory, and device memory holds only split twiddle tables.  Its
results equal the in-HBM pp_ntt bit for bit, forward and inverse, at every
pass count; the device memory it allocates is a small fraction of the data
(and nothing on a repeated call)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import host

pytestmark = pytest.mark.gpu


def _pinned_copy(P, x):
    h = P.empty_pinned(x.shape[0])
    h.copy_(x.cpu())
    return h


@pytest.mark.parametrize("lg", [1, 5, 11, 12, 17, 20, 23, 24])
@pytest.mark.parametrize("inverse", [False, True])
def test_out_of_core_equals_in_hbm_transform(pp, cuda, lg, inverse):
    P = pp.ppfr
    n = 1 << lg
    x = pp.random_fr(n, 0x00C0 + lg + (100 if inverse else 0))
    want = host(pp.ntt(x, inverse))
    hin = _pinned_copy(P, x)
    hout, hs = P.empty_pinned(n), P.empty_pinned(n)
    before = P.device_alloc_bytes()
    P.ntt_out_of_core(hin, inverse, out=hout, scratch=hs)
    cuda.cuda.synchronize()
    first = P.device_alloc_bytes() - before
    got = hout.numpy().view(np.uint64).reshape(-1, 4)
    bad = np.nonzero((got != want).any(axis=1))[0]
    assert bad.size == 0, bad[:5]
    assert (hin.numpy().view(np.uint64).reshape(-1, 4) == host(x)).all()  # input untouched
    if lg >= 20:
        assert first < (32 * n) // 64, first  # tables only: far below the data's size
    # a second call finds its tables and allocates nothing
    before = P.device_alloc_bytes()
    P.ntt_out_of_core(hin, inverse, out=hout, scratch=hs)
    cuda.cuda.synchronize()
    assert P.device_alloc_bytes() == before
    assert (hout.numpy().view(np.uint64).reshape(-1, 4) == want).all()


def test_out_of_core_2p26(pp, cuda):
    P = pp.ppfr
    n = 1 << 26
    x = pp.random_fr(n, 0x00C26)
    want = pp.ntt(x)
    hin = _pinned_copy(P, x)
    del x
    hout = P.ntt_out_of_core(hin)
    cuda.cuda.synchronize()
    assert (hout.numpy().view(np.uint64).reshape(-1, 4) == host(want)).all()


def test_out_of_core_refuses_bad_buffers(pp, cuda):
    import torch

    P = pp.ppfr
    n = 1 << 12
    a, b = P.empty_pinned(n), P.empty_pinned(n)
    with pytest.raises(P.PPError):
        P.ntt_out_of_core(a, out=b, scratch=a)  # not three distinct buffers
    pageable = torch.empty((n, 4), dtype=torch.int64)
    with pytest.raises(P.PPError):
        P.ntt_out_of_core(pageable, out=a, scratch=b)


# ------------------------------------------------------- out-of-core LDE
# pp_lde_out_of_core against the in-HBM pp_lde, every mode: one pass
# (2^(lg + lambda) <= 2^11), two and three passes, both placements of the
# evaluations form's coefficients (which depend on the pass count), and the
# BASELINE sizes 2^22 (lambda 2, 3) and 2^24 (lambda 2).
@pytest.mark.parametrize("lg,lam", [(4, 2), (9, 2), (10, 3), (12, 2), (15, 3), (18, 2), (20, 3), (22, 2),
                                    (22, 3), (24, 2)])
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_lde_out_of_core_equals_in_hbm(pp, cuda, lg, lam, mode):
    P = pp.ppfr
    n = 1 << lg
    x = pp.random_fr(n, 0x0D00 + 7 * lg + lam + 31 * mode)
    want = host(pp.lde(x, lam, mode))
    hin = _pinned_copy(P, x)
    hout, hs = P.empty_pinned(n << lam), P.empty_pinned(n << lam)
    before = P.device_alloc_bytes()
    P.lde_out_of_core(hin, lam, mode, out=hout, scratch=hs)
    cuda.cuda.synchronize()
    first = P.device_alloc_bytes() - before
    got = hout.numpy().view(np.uint64).reshape(-1, 4)
    bad = np.nonzero((got != want).any(axis=1))[0]
    assert bad.size == 0, bad[:5]
    assert (hin.numpy().view(np.uint64).reshape(-1, 4) == host(x)).all()  # input untouched
    if lg >= 20:
        assert first < (32 * n) // 64, first  # tables only: far below the data's size


def test_lde_out_of_core_refuses_bad_buffers(pp, cuda):
    P = pp.ppfr
    n = 1 << 12
    a, b = P.empty_pinned(n), P.empty_pinned(n << 2)
    with pytest.raises(P.PPError):
        P.lde_out_of_core(a, 2, 0, out=b, scratch=b)  # not three distinct buffers
    with pytest.raises(P.PPError):
        P.lde_out_of_core(a, 9, 0, out=b, scratch=P.empty_pinned(n << 2))  # lambda > 8
