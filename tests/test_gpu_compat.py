"""The reference-compatible C++ host layer (SyncedMemory, Ntt/Intt,
accumulate_mul_poly, evaluate, poly_div_poly, our_ntt, standard4_ntt,
our_lde, naive_lde) driven like the reference's own drivers, on raw files of
Montgomery elements, checked against the oracle."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

DRIVER = os.path.join(ROOT, "ppopp26-artifact_gb300", "pp_compat_driver")


def run(*args):
    r = subprocess.run([DRIVER, *map(str, args)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def load(path, n):
    return np.fromfile(path, dtype=np.uint64).reshape(n, 4)


@pytest.mark.parametrize("lg", [1, 10, 16])
def test_miss_ops_driver(pp, O, cuda, tmp_path, lg):
    n = 1 << lg
    x = O.random_fr(n, 4000 + lg)
    x.tofile(tmp_path / "in.bin")
    run("miss_ops", lg, tmp_path / "in.bin", tmp_path)
    assert O.first_diff(load(tmp_path / "gp.bin", n), O.gp_prefix(x)) == -1
    incl = O.gp_prefix(x)
    incl = np.array([O.fr_mul(incl[i], x[i]) for i in range(n)]) if n <= 1024 else None
    if incl is not None:
        assert O.first_diff(load(tmp_path / "gp_incl.bin", n), incl) == -1
    pt = np.array([123456789, 987654321, 1122334455, 6677889900], np.uint64)
    assert (load(tmp_path / "eval.bin", 1)[0] == O.evaluate(x, pt)).all()
    c = np.array([123456789123456789, 987654321987654321, 1122334455667788, 1122334455667788], np.uint64)
    assert O.first_diff(load(tmp_path / "div.bin", n), O.div_xplusc(x, c)) == -1


@pytest.mark.parametrize("lg", [3, 12, 20])
def test_ntt_driver_checks(pp, O, cuda, tmp_path, lg):
    n = 1 << lg
    x = O.random_fr(n, 5000 + lg)
    x.tofile(tmp_path / "in.bin")
    out = run("ntt", lg, tmp_path / "in.bin", tmp_path / "out.bin")
    assert "our_ntt: ok, standard4_ntt: ok, intt round trip: ok" in out
    assert O.first_diff(load(tmp_path / "out.bin", n), O.ntt(x)) == -1


@pytest.mark.parametrize("lg,lam", [(8, 2), (16, 3)])
def test_lde_driver(pp, O, cuda, tmp_path, lg, lam):
    n = 1 << lg
    x = O.random_fr(n, 6000 + lg)
    x.tofile(tmp_path / "in.bin")
    run("lde", lg, lam, tmp_path / "in.bin", tmp_path / "out.bin")
    assert O.first_diff(load(tmp_path / "out.bin", n << lam), O.lde_coeffs(x, lam)) == -1
    run("lde", lg, lam, tmp_path / "in.bin", tmp_path / "out2.bin", "naive")
    assert O.first_diff(load(tmp_path / "out2.bin", n << lam), O.lde_spread(x, lam)) == -1


GOLD = os.path.join(ROOT, "tests", "golden", "constraints.npz")


@pytest.mark.parametrize("n", [7, 64])
def test_quotient_driver_matches_golden(pp, O, cuda, tmp_path, n):
    """The three permutation-term entry points, called in sequence on one
    result buffer as the prover does, through the C++ layer."""
    g = np.load(GOLD)
    t = "perm_n%d/" % n
    for k in g.files:
        if k.startswith(t):
            np.ascontiguousarray(g[k]).tofile(tmp_path / (k[len(t):] + ".bin"))
    run("quotient", n, tmp_path)
    # identity writes result, copy and term-one add to it
    want = g[t + "identity"]
    w = [g[t + k] for k in ("w_l", "w_r", "w_o", "w_4")]
    sig = [g[t + k] for k in ("left_sigma", "right_sigma", "out_sigma", "fourth_sigma")]
    want = O.quotient_copy(sig, g[t + "mod"], w, g[t + "z_next"], g[t + "alpha"][0], g[t + "beta"][0],
                           g[t + "gamma"][0], want)
    want = O.quotient_term_one(g[t + "z"], g[t + "l1"], g[t + "one"][0], want)
    assert np.array_equal(load(tmp_path / "quotient_out.bin", n), want)


@pytest.mark.parametrize("case", ["gate_rand_a5_n64", "gate_small_a5_n33", "gate_rand_a2_n16"])
def test_gate_driver_matches_golden(pp, cuda, tmp_path, case):
    g = np.load(GOLD)
    t = case + "/"
    for k in g.files:
        if k.startswith(t) and not k.endswith("SBOX_ALPHA"):
            np.ascontiguousarray(g[k]).tofile(tmp_path / (k[len(t):] + ".bin"))
    n = g[t + "out"].shape[0]
    run("gate", n, int(g[t + "SBOX_ALPHA"][0]), tmp_path)
    assert np.array_equal(load(tmp_path / "gate_out.bin", n), g[t + "out"])


@pytest.mark.parametrize("case", ["rand_n64", "edge_n16"])
def test_msm_driver_matches_blst(pp, cuda, tmp_path, case):
    """multi_scalar_mult through the C++ layer (PLONK/utils/function.cuh:144)."""
    g = np.load(os.path.join(ROOT, "tests", "golden", "msm.npz"))
    pts, sc = g[case + "/points"], g[case + "/scalars"]
    pts.tofile(tmp_path / "p.bin")
    sc.tofile(tmp_path / "s.bin")
    run("msm", len(pts), tmp_path / "p.bin", tmp_path / "s.bin", tmp_path / "o.bin")
    o = np.fromfile(tmp_path / "o.bin", dtype=np.uint64).reshape(3, 6)
    assert np.array_equal(np.concatenate([o[0], o[1]]), g[case + "/out"])


@pytest.mark.parametrize("n", [2, 64, 1000])
def test_fieldops_driver(pp, O, cuda, tmp_path, n):
    """add_mod ... make_tensor and gt_zkp through the C++ layer."""
    a = O.random_fr(n, 0x5100 + n)
    b = O.random_fr(n, 0x5200 + n)
    b[1] = 0  # division by 0 gives 0
    s = O.random_fr(1, 0x5300 + n)
    a.tofile(tmp_path / "a.bin")
    b.tofile(tmp_path / "b.bin")
    s.tofile(tmp_path / "s.bin")
    out = run("fieldops", n, tmp_path)
    gt_ab = [int(t) for t in out.split("gt ")[1].split()[:2]]
    big = lambda x: sum(int(w) << (64 * k) for k, w in enumerate(x.ravel()))  # noqa: E731
    assert gt_ab == [int(big(a) > big(b)), int(big(b) > big(a))]
    f = lambda name, m=n: load(tmp_path / (name + ".bin"), m)  # noqa: E731
    inv = lambda y: O.fr_inv(y)  # noqa: E731  (inverse of 0 is 0)
    for i in range(n):
        assert (f("add")[i] == O.fr_add(a[i], b[i])).all()
        assert (f("sub")[i] == O.fr_sub(a[i], b[i])).all()
        assert (f("mul")[i] == O.fr_mul(a[i], b[i])).all()
        q = O.fr_mul(a[i], inv(b[i]))
        assert (f("div")[i] == q).all() and (f("div_in_place")[i] == q).all()
        assert (f("add_scalar")[i] == O.fr_add(a[i], s[0])).all()
        assert (f("div_scalar")[i] == O.fr_mul(a[i], inv(s[0]))).all()
        assert (f("mul_scalar_in_place")[i] == O.fr_mul(a[i], s[0])).all()
        assert (f("neg")[i] == O.fr_neg(a[i])).all()
        assert (f("inv")[i] == inv(b[i])).all()
        assert (f("exp5")[i] == O.fr_pow(a[i], 5)).all()
        assert (f("seq")[i] == O.fr_pow(s[0], i)).all()
        assert (f("rep")[i] == s[0]).all()
    pad = f("pad", 2 * n)
    assert (pad[:n] == a).all() and not pad[n:].any()
    assert (f("cat", 2 * n) == np.concatenate([a, b])).all()
    assert (f("slice", n // 2) == a[n - n // 2:]).all()
    tensor = f("tensor", 4 * n)
    assert (tensor[:, 0] == a.ravel()).all() and not tensor[:, 1:].any()
