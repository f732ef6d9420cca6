"""The reference's own ``miss_ops.cu``, unmodified, built against this library
and run on the GPU.

The file is copied alone into a scratch directory and compiled with
``ppopp26-artifact_gb300/host/ref_include`` on the include path, so its
``#include "caffe/interface.hpp"`` and ``#include "PLONK/utils/function.cuh"``
resolve to this library's SyncedMemory, operator entry points and host field
element.  Two programs are linked against ``libppcompat.so`` / ``libppfr.so``:

* the file as it is, whose ``main`` (miss_ops.cu:88-204) reads
  ``../../input.bin`` (2^22 elements), runs the blst baselines and the three
  GPU operators three times each, and prints their times;
* the file with ``main`` renamed, plus ``tests/dropin_miss_ops_harness.cpp``,
  which writes every operator's output so that it can be checked against the
  oracle.

Needs the staged reference copy (``make -C oracle stage REF_CHECKOUT=...``);
skipped where it is absent.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

PKG = os.path.join(ROOT, "ppopp26-artifact_gb300")
STAGED_MISS_OPS = os.path.join(ROOT, "oracle", "_ref", "src", "miss_ops.cu")
needs_staged = pytest.mark.skipif(not os.path.exists(STAGED_MISS_OPS), reason="no staged reference copy")


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _build(tmp, name, extra_src=(), defines=()):
    src = os.path.join(tmp, "miss_ops.cu")
    shutil.copy(STAGED_MISS_OPS, src)
    exe = os.path.join(tmp, name)
    inc = ["-I" + os.path.join(PKG, "host", "ref_include"), "-I" + os.path.join(PKG, "host"),
           "-I" + os.path.join(ROOT, "include")]
    flags = [_nvcc(), "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a", *inc]
    obj = os.path.join(tmp, name + "_miss_ops.o")
    r = subprocess.run([*flags, *defines, "-c", src, "-o", obj], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    r = subprocess.run([*flags, obj, *extra_src, "-o", exe, "-L" + PKG, "-lppcompat", "-lppfr",
                        "-Xlinker", "-rpath=" + PKG], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def _load(path, n):
    a = np.fromfile(path, dtype=np.uint64)
    assert a.size == 4 * n, (path, a.size)
    return a.reshape(n, 4)


@needs_staged
@pytest.mark.parametrize("lg", [4, 12, 20])
def test_reference_miss_ops_outputs(pp, O, cuda, tmp_path, lg):
    exe = _build(str(tmp_path), "dropin", [os.path.join(ROOT, "tests", "dropin_miss_ops_harness.cpp")],
                 ["-Dmain=reference_miss_ops_main"])
    n = 1 << lg
    a = O.random_fr(n, 0xD0000 + lg)
    x = O.random_fr(1, 0xD1000 + lg)
    c = O.random_fr(1, 0xD2000 + lg)
    for name, v in (("in", a), ("x", x), ("c", c)):
        v.tofile(tmp_path / (name + ".bin"))
    out = str(tmp_path / "out")
    r = subprocess.run([exe, str(lg), str(tmp_path / "in.bin"), str(tmp_path / "x.bin"), str(tmp_path / "c.bin"),
                        out], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "dropin ok" in r.stdout, r.stdout + r.stderr
    # the reference's blst loops, run on this library's host field element
    assert O.first_diff(_load(out + ".naive_gp", n), O.naive_gp(a)) == -1
    q, _ = O.naive_div(a, c[0])
    assert O.first_diff(_load(out + ".naive_div", n - 1), q) == -1
    # this library's GPU operators behind the reference's entry points
    assert O.first_diff(_load(out + ".gp", n), O.gp_prefix(a)) == -1
    assert (_load(out + ".eval", 1)[0] == O.evaluate(a, x[0])).all()
    assert O.first_diff(_load(out + ".div", n), O.div_xplusc(a, c[0])) == -1


@needs_staged
def test_reference_miss_ops_main_runs(pp, O, cuda, tmp_path):
    exe = _build(str(tmp_path), "miss_ops")
    O.random_fr(1 << 22, 0xD3000).tofile(tmp_path / "input.bin")  # miss_ops.cu:94: ../../input.bin
    wd = tmp_path / "build" / "miss_ops"
    wd.mkdir(parents=True)
    r = subprocess.run([exe], cwd=str(wd), capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    for tag in ("[naive_gp]", "[ours_gp]", "[ours_eval]", "[naive_div]", "[ours_div]"):
        assert r.stdout.count(tag + " execution time") == 3, tag
