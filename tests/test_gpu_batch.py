"""Batch plans: a mix of NTT, INTT, the three LDE forms and grand products of
uneven sizes in one plan gives, bit for bit, the single-call results, run
directly and replayed from a captured CUDA graph."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import host

pytestmark = pytest.mark.gpu


def _mix(pp, seed):
    P = pp.ppfr
    rng = np.random.default_rng(seed)
    jobs, refs = [], []
    spec = [(P.JOB_NTT, 12, 0), (P.JOB_INTT, 14, 0), (P.JOB_NTT, 3, 0), (P.JOB_LDE_COEFFS, 10, 2),
            (P.JOB_LDE_EVALS, 11, 2), (P.JOB_LDE_SPREAD, 9, 3), (P.JOB_GP, 13, 0), (P.JOB_NTT, 17, 0),
            (P.JOB_INTT, 20, 0), (P.JOB_LDE_COEFFS, 16, 3), (P.JOB_GP, 10, 0)]
    for i, (kind, lg, lam) in enumerate(spec):
        x = P.random_fr(1 << lg, 1000 + 17 * i + int(rng.integers(0, 9)))
        out = P.empty(1 << (lg + lam))
        jobs.append((kind, x, out, lam))
        if kind == P.JOB_NTT:
            refs.append(P.ntt(x))
        elif kind == P.JOB_INTT:
            refs.append(P.ntt(x, True))
        elif kind == P.JOB_GP:
            refs.append(P.gp_prefix_(x.clone()))
        else:
            mode = {P.JOB_LDE_COEFFS: P.LDE_COEFFS, P.JOB_LDE_EVALS: P.LDE_EVALS,
                    P.JOB_LDE_SPREAD: P.LDE_SPREAD}[kind]
            refs.append(P.lde(x, lam, mode))
    return jobs, refs


def test_batch_matches_single_calls(pp, O, cuda):
    torch = cuda
    jobs, refs = _mix(pp, 1)
    b = pp.ppfr.Batch(jobs)
    info = b.info()
    assert info["launches"] <= 8, info  # a few levels + 2 grand-product launches, not ~30
    b.run()
    torch.cuda.synchronize()
    for (kind, x, out, lam), ref in zip(jobs, refs):
        assert torch.equal(out, ref), (kind, x.shape[0], lam)
    # the small NTT against the oracle too
    kind, x, out, lam = jobs[0]
    assert O.first_diff(host(out), O.ntt(host(x))) == -1
    b.close()


def test_batch_graph_replay(pp, cuda):
    torch = cuda
    jobs, refs = _mix(pp, 2)
    b = pp.ppfr.Batch(jobs)
    b.capture()
    for _ in range(3):
        for _, _, out, _ in jobs:
            out.zero_()
        b.run()
        torch.cuda.synchronize()
        for (kind, x, out, lam), ref in zip(jobs, refs):
            assert torch.equal(out, ref), (kind, x.shape[0], lam)
    b.close()


def test_batch_more_jobs_than_one_launch_carries(pp, cuda):
    """300 small jobs: each level needs three launches of at most 128 job
    passes; every result equals its single call."""
    torch = cuda
    P = pp.ppfr
    rng = np.random.default_rng(77)
    jobs, refs = [], []
    for i in range(300):
        lg = int(rng.integers(3, 12))
        inverse = bool(i & 1)
        x = P.random_fr(1 << lg, 5000 + i)
        jobs.append((P.JOB_INTT if inverse else P.JOB_NTT, x, P.empty(1 << lg), 0))
        refs.append(P.ntt(x, inverse))
    b = P.Batch(jobs)
    assert b.info()["launches"] >= 3
    for _ in range(2):
        b.run()
        torch.cuda.synchronize()
        for (_, _, out, _), ref in zip(jobs, refs):
            assert torch.equal(out, ref)
    b.close()
