"""Host-resident transforms (pp_ntt_host / pp_lde_host, the GB300 form of the
reference's our_ntt / our_lde, ntt.cu:979-1037 and lde.cu:1267-1365): input and
output in page-locked host memory, read and written by the first and last
passes directly.  Results must equal the device-resident operators bit for bit
and the oracle; buffers that are not page-locked are refused on the host."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dev, host

pytestmark = pytest.mark.gpu


def pinned_from(torch, a):
    t = torch.empty((a.shape[0], 4), dtype=torch.int64, pin_memory=True)
    t.copy_(torch.from_numpy(a.view(np.int64).reshape(-1, 4)))
    return t


def as_u64(t):
    return t.numpy().view(np.uint64).reshape(-1, 4)


@pytest.mark.parametrize("lg", [0, 1, 2, 3, 7, 11, 12, 16, 20])
@pytest.mark.parametrize("inverse", [False, True])
def test_ntt_host_equals_device_and_oracle(pp, O, cuda, lg, inverse):
    import torch
    P = pp.ppfr
    x = O.random_fr(1 << lg, 900 + lg)
    hx = pinned_from(torch, x)
    out = P.ntt_host(hx, inverse=inverse)
    torch.cuda.synchronize()
    want = host(P.ntt(dev(x), inverse=inverse))
    assert np.array_equal(as_u64(out), want)
    if lg <= 16:
        assert O.first_diff(as_u64(out), O.ntt(x, inverse=inverse)) == -1
    assert np.array_equal(as_u64(hx), x)  # input untouched


def test_ntt_host_in_place(pp, O, cuda):
    import torch
    P = pp.ppfr
    x = O.random_fr(1 << 18, 77)
    hx = pinned_from(torch, x)
    P.ntt_host(hx, out=hx)
    torch.cuda.synchronize()
    assert np.array_equal(as_u64(hx), host(P.ntt(dev(x))))
    P.ntt_host(hx, inverse=True, out=hx)
    torch.cuda.synchronize()
    assert np.array_equal(as_u64(hx), x)


def test_ntt_host_full_size(pp, cuda):
    import torch
    P = pp.ppfr
    n = 1 << 24
    d = P.random_fr(n, 0x5EED0018)
    hx = torch.empty((n, 4), dtype=torch.int64, pin_memory=True)
    hx.copy_(d)
    out = P.ntt_host(hx)
    torch.cuda.synchronize()
    assert torch.equal(out, P.ntt(d).cpu())


@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("lg,lam", [(4, 1), (10, 2), (12, 3), (16, 2)])
def test_lde_host_equals_device(pp, O, cuda, mode, lg, lam):
    import torch
    P = pp.ppfr
    x = O.random_fr(1 << lg, 31 * lg + lam)
    out = P.lde_host(pinned_from(torch, x), lam, mode)
    torch.cuda.synchronize()
    assert np.array_equal(as_u64(out), host(P.lde(dev(x), lam, mode)))
    if lg <= 12:
        ref = {0: O.lde_coeffs, 1: O.lde_evals, 2: O.lde_spread}[mode](x, lam)
        assert O.first_diff(as_u64(out), ref) == -1


def test_host_forms_refuse_unpinned_and_device_buffers(pp, cuda):
    import torch
    P = pp.ppfr
    n = 1 << 10
    pageable = torch.zeros((n, 4), dtype=torch.int64)
    pinned = torch.zeros((n, 4), dtype=torch.int64, pin_memory=True)
    with pytest.raises(P.PPError) as e:
        P.ntt_host(pageable, out=pinned)
    assert e.value.status == 1
    with pytest.raises(P.PPError) as e:
        P.ntt_host(pinned, out=pageable)
    assert e.value.status == 1
    with pytest.raises(P.PPError) as e:
        P.lde_host(pageable, 1, out=torch.zeros((2 * n, 4), dtype=torch.int64, pin_memory=True))
    assert e.value.status == 1
    # a device pointer is not host memory either (called through the ABI directly)
    L = P.lib()
    d = P.empty(n)
    import ctypes
    st = L.pp_ntt_host(ctypes.c_void_p(d.data_ptr()), ctypes.c_void_p(pinned.data_ptr()), 10, 0, None)
    assert st == 1
    torch.cuda.synchronize()


@pytest.mark.parametrize("lg,count", [(0, 1), (5, 2), (12, 7), (20, 5)])
@pytest.mark.parametrize("inverse", [False, True])
def test_ntt_host_many(pp, O, cuda, lg, count, inverse):
    """pp_ntt_host_many: every polynomial equals its own device transform,
    with the three device buffers reused (count > 3) and some polynomials in
    place (h_out[j] == h_in[j])."""
    import torch
    P = pp.ppfr
    xs = [O.random_fr(1 << lg, 0x4A00 + 16 * lg + j) for j in range(count)]
    hins = [pinned_from(torch, x) for x in xs]
    outs = [h if j % 3 == 1 else P.empty_pinned(1 << lg) for j, h in enumerate(hins)]
    s = torch.cuda.Stream()
    P.ntt_host_many(hins, inverse=inverse, outs=outs, stream=s)
    s.synchronize()
    for j, x in enumerate(xs):
        want = host(P.ntt(dev(x), inverse=inverse))
        assert np.array_equal(as_u64(outs[j]), want), j
        if j % 3 != 1:
            assert np.array_equal(as_u64(hins[j]), x)  # input untouched
    if lg <= 12:
        assert O.first_diff(as_u64(outs[-1]), O.ntt(xs[-1], inverse=inverse)) == -1


def test_ntt_host_many_refusals(pp, O, cuda):
    import torch
    P = pp.ppfr
    n = 1 << 10
    x = O.random_fr(n, 0x4B00)
    good = [pinned_from(torch, x) for _ in range(3)]
    outs = [torch.zeros((n, 4), dtype=torch.int64, pin_memory=True) for _ in range(3)]
    assert P.ntt_host_many([], outs=[]) == []  # count 0
    bad_out = outs[:2] + [torch.zeros((n, 4), dtype=torch.int64)]  # pageable
    with pytest.raises(P.PPError) as e:
        P.ntt_host_many(good, outs=bad_out)
    assert e.value.status == 1
    torch.cuda.synchronize()
    # refused before any copy was queued: the good outputs are untouched
    assert not outs[0].any() and not outs[1].any()
    P.ntt_host_many(good, outs=outs)
    torch.cuda.synchronize()
    want = host(P.ntt(dev(x)))
    assert all(np.array_equal(as_u64(o), want) for o in outs)
