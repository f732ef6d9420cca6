"""The device field code (csrc/fr.cuh) compiled for the host: its PTX
carry-chain primitives run as exact host emulations, so every Montgomery
multiply variant, add, sub, pow and inverse is checked against the oracle on
the CPU."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import ROOT


def test_field_code_matches_oracle(tmp_path):
    exe = str(tmp_path / "fr_host_check")
    objs = []
    for src, lang in (("tests/fr_host_check.cpp", "c++"), ("oracle/pp_oracle.c", "c")):
        obj = str(tmp_path / (os.path.basename(src) + ".o"))
        cc = "g++" if lang == "c++" else "gcc"
        std = ["-std=c++17"] if lang == "c++" else ["-std=gnu11"]
        subprocess.run([cc, "-O2", "-fopenmp", *std, "-c", os.path.join(ROOT, src), "-o", obj], check=True)
        objs.append(obj)
    subprocess.run(["g++", "-fopenmp", *objs, "-o", exe], check=True)
    r = subprocess.run([exe, "20000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
