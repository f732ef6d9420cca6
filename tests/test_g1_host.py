"""The device G1 code (csrc/g1.cuh over csrc/fq.cuh) compiled for the host,
its carry chains emulated: point addition, doubling and their equal-x cases
against the oracle, and small multi-scalar sums against the blst golden
vectors (tests/golden/msm.npz)."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

GOLD = os.path.join(ROOT, "tests", "golden", "msm.npz")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    d = tmp_path_factory.mktemp("g1")
    objs = []
    for src, cc, std in (("tests/g1_host_check.cpp", "g++", "-std=c++17"),
                         ("oracle/pp_oracle.c", "gcc", "-std=gnu11"),
                         ("oracle/pp_oracle_g1.c", "gcc", "-std=gnu11")):
        obj = str(d / (os.path.basename(src) + ".o"))
        subprocess.run([cc, "-O2", "-fopenmp", std, "-c", os.path.join(ROOT, src), "-o", obj], check=True)
        objs.append(obj)
    out = str(d / "g1_host_check")
    subprocess.run(["g++", "-fopenmp", *objs, "-o", out], check=True)
    return out


def test_point_formulas_match_oracle(exe):
    r = subprocess.run([exe, "add", "64"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "mismatches 0" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("case", ["rand_n7", "edge_n16", "cancel_n2"])
def test_small_msm_matches_blst(exe, tmp_path, case):
    g = np.load(GOLD)
    pts, sc = g[case + "/points"], g[case + "/scalars"]
    pts.tofile(tmp_path / "p.bin")
    sc.tofile(tmp_path / "s.bin")
    r = subprocess.run([exe, "msm", str(tmp_path / "p.bin"), str(tmp_path / "s.bin"), str(len(pts)),
                        str(tmp_path / "o.bin")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.fromfile(tmp_path / "o.bin", dtype=np.uint64), g[case + "/out"])
