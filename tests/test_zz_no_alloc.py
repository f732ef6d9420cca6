"""pp_eval_noalloc: evaluation for callers that must not allocate device memory
during a call (a process whose device memory is all held by its own pool; a
latency-critical loop that cannot take the device-wide synchronisation of
cudaMalloc/cudaFree).  Its scratch is a static device array, so it is checked
through the C ABI against the allocating pp_eval on two calls in a row, the
second smaller than the first so that leftovers of the first would show.

This file is collected last on purpose; it must also pass on its own in a
fresh process."""
from __future__ import annotations

import ctypes

import pytest

from conftest import host

pytestmark = pytest.mark.gpu

PP_E_UNSUPPORTED = 5
MAX_N = 1 << 22


def _fn(pp):
    f = pp.ppfr.lib().pp_eval_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def test_eval_noalloc_matches_pp_eval(pp, O, cuda):
    torch = cuda
    f = _fn(pp)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for n, seed in ((MAX_N, 11), (12345, 12)):
        p = pp.random_fr(n, seed)
        x = pp.random_fr(1, seed + 1000)
        y_noalloc = pp.ppfr.empty(1)
        y_ref = pp.ppfr.empty(1)
        st = f(p.data_ptr(), n, x.data_ptr(), y_noalloc.data_ptr(), stream)
        assert st == 0, pp.ppfr.lib().pp_last_error()
        pp.evaluate(p, x, out=y_ref)
        torch.cuda.synchronize()
        assert (host(y_noalloc) == host(y_ref)).all(), n
    # the small case against the oracle as well
    assert (host(y_noalloc)[0] == O.evaluate(host(p), host(x)[0])).all()


def test_eval_noalloc_does_not_allocate(pp, cuda):
    """The library's own count of the device allocations it requests does not
    move across the calls, set-up call included.  (Device-wide free memory is
    not used: other allocations on the device would change it.)"""
    torch = cuda
    f = _fn(pp)
    L = pp.ppfr.lib()
    L.pp_device_alloc_count.restype = ctypes.c_uint64
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = pp.random_fr(1 << 20, 21)
    x = pp.random_fr(1, 22)
    y = pp.ppfr.empty(1)
    torch.cuda.synchronize()
    before = L.pp_device_alloc_count()
    for _ in range(4):
        assert f(p.data_ptr(), 1 << 20, x.data_ptr(), y.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    assert L.pp_device_alloc_count() == before
    # the counter does see allocations: with the cached workspaces dropped,
    # the allocating form takes a new one
    pp.ppfr.release()
    pp.evaluate(p, x, out=y)
    torch.cuda.synchronize()
    assert L.pp_device_alloc_count() > before


def test_eval_noalloc_rejects_oversize(pp, cuda):
    f = _fn(pp)
    p = pp.random_fr(16, 31)
    x = pp.random_fr(1, 32)
    y = pp.ppfr.empty(1)
    st = f(p.data_ptr(), MAX_N + 1, x.data_ptr(), y.data_ptr(), None)
    assert st == PP_E_UNSUPPORTED
    assert b"2^22" in pp.ppfr.lib().pp_last_error()
