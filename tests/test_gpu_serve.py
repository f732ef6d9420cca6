"""The serving loop: a bundle's results are the same alone and in a mix of
concurrently admitted bundles, equal to the plain operators on the same
inputs (and to the oracle on a small case); admission respects the memory
budget; queued bundles can be cancelled; waits are bounded."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import dev, host

pytestmark = pytest.mark.gpu

LAM = 2


def fetch(P, r, lg):
    n = 1 << lg
    out = {"lde": [P.copy_to_host(r.d_lde[j], n << LAM) for j in range(3)],
           "z": P.copy_to_host(r.d_z, n), "q": P.copy_to_host(r.d_quotient, n),
           "evals": P.copy_to_host(r.d_evals, 6),
           "w": [P.copy_to_host(r.d_w[j], n) for j in range(3)],
           "sigma": [P.copy_to_host(r.d_sigma[j], n) for j in range(3)],
           "params": P.copy_to_host(r.d_params, 12)}
    return out


def same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(
        a["lde"] + [a["z"], a["q"], a["evals"]], b["lde"] + [b["z"], b["q"], b["evals"]]))


def test_bundle_alone_equals_plain_operators_and_oracle(pp, O, cuda):
    P = pp.ppfr
    srv = P.Server(budget_bytes=4 << 30, slots=4, min_lg=6, max_lg=12, lam=LAM)
    lg = 8
    t = srv.submit(lg, seed=77)
    r = srv.wait(t)
    res = fetch(P, r, lg)
    srv.release(t)
    srv.close()
    n = 1 << lg
    w, s, prm = res["w"], res["sigma"], res["params"]
    # the plain operators on the same inputs
    for j in range(3):
        assert np.array_equal(host(P.lde(dev(w[j]), LAM, P.LDE_COEFFS)), res["lde"][j])
    z = P.gp_perm([dev(x) for x in w], [dev(x) for x in s], dev(prm[:5]))
    assert np.array_equal(host(z), res["z"])
    # the oracle, independently
    assert O.first_diff(res["lde"][0], O.lde_coeffs(w[0], LAM)) == -1
    ks = [prm[2], prm[3], prm[4]]
    assert O.first_diff(res["z"], O.gp_perm(w, s, prm[0], prm[1], ks)) == -1
    polys = w + s
    for k in range(6):
        assert (res["evals"][k] == O.evaluate(polys[k], prm[6 + k])).all(), k
    # the polynomial divided is the seventh input block, regenerated from the seed
    divp = O.random_fr(7 * n, 77)[6 * n:7 * n]
    assert O.first_diff(res["q"], O.div_xplusc(divp, prm[5])) == -1


def test_bundle_same_alone_and_in_mix(pp, cuda):
    P = pp.ppfr
    srv = P.Server(budget_bytes=8 << 30, slots=4, min_lg=8, max_lg=16, lam=LAM)
    t = srv.submit(12, seed=4242)
    alone = fetch(P, srv.wait(t), 12)
    srv.release(t)
    srv.reset_stats()
    rng = np.random.default_rng(5)
    tickets = []
    for i in range(16):
        lg = int(rng.integers(8, 17))
        tickets.append((srv.submit(lg, seed=1000 + i), lg, None))
        if i == 7:
            tickets.append((srv.submit(12, seed=4242), 12, "probe"))
    got = None
    for tk, lg, tag in tickets:
        r = srv.wait(tk)
        assert r.status == 0
        if tag == "probe":
            got = fetch(P, r, lg)
        srv.release(tk)
    st = srv.stats()
    srv.close()
    assert got is not None and same(alone, got)
    assert st["completed"] == 17
    assert st["max_concurrent"] > 1 and st["admitted_while_busy"] > 0, st
    assert st["p99_ms"] >= st["p50_ms"] > 0


def test_budget_admission_and_cancel(pp, cuda):
    P = pp.ppfr
    lg = 16
    one = (20 * (1 << lg) + 24) * 32  # one bundle's buffers at lambda = 2
    srv = P.Server(budget_bytes=int(one * 1.5), slots=4, min_lg=lg, max_lg=lg, lam=LAM)
    ts = [srv.submit(lg, seed=9000 + i) for i in range(4)]
    assert srv.cancel(ts[3]) in (0, 7)  # queued -> cancelled; already admitted -> busy
    for t in ts[:3]:
        r = srv.wait(t)
        assert r.status == 0
        srv.release(t)
    st = srv.stats()
    assert st["budget_peak"] <= int(one * 1.5)
    assert st["max_concurrent"] == 1  # the budget holds one bundle at a time
    status = srv.wait_status(ts[3], 1000)
    assert status in (0, 6)  # done or PP_E_CANCELLED
    srv.close()


def test_work_cap_admission(pp, cuda):
    """With the running work capped below two bundles' work, bundles run one
    at a time (the cap never holds back a bundle when nothing runs), and the
    results equal those of the uncapped server."""
    P = pp.ppfr
    lg = 14
    one = P.bundle_work(lg, LAM)
    assert one == 3 * ((4 << lg) // 2 * (lg + LAM) + (1 << lg)) + 23 * (1 << lg)
    outs = []
    for cap in (one + one // 2, 0):
        srv = P.Server(budget_bytes=4 << 30, slots=4, min_lg=lg, max_lg=lg, lam=LAM, max_inflight_mm=cap)
        ts = [srv.submit(lg, seed=9100 + i) for i in range(4)]
        res = []
        for t in ts:
            r = srv.wait(t)
            assert r.status == 0
            res.append(fetch(P, r, lg))
            srv.release(t)
        st = srv.stats()
        if cap:
            assert st["max_concurrent"] == 1
        outs.append(res)
        srv.close()
    assert all(same(a, b) for a, b in zip(*outs))


def test_wait_is_bounded(pp, cuda):
    P = pp.ppfr
    srv = P.Server(budget_bytes=2 << 30, slots=1, min_lg=14, max_lg=14, lam=LAM)
    ts = [srv.submit(14, seed=i) for i in range(6)]
    # the last bundle is queued behind five others on one slot: a 0 ms wait times out
    assert srv.wait_status(ts[-1], 0) in (4, 0)  # PP_E_TIMEOUT (or already done)
    for t in ts:
        srv.wait(t)
        srv.release(t)
    srv.close()
