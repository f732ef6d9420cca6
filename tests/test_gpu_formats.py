"""Data formats either side of the path: raw element files (the reference's
input.bin layout), Montgomery encoding/decoding on the device (to_mont /
to_base, PLONK/utils/function.cu:5-21) and the canonical-form count, through
the Python front end and through the C++ layer's read_file / writeToFile."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, dev, host

pytestmark = pytest.mark.gpu

R = 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001
DRIVER = os.path.join(ROOT, "ppopp26-artifact_gb300", "pp_compat_driver")


def ints(a):
    return [sum(int(w) << (64 * k) for k, w in enumerate(row)) for row in a]


def limbs(vals):
    return np.array([[(v >> (64 * k)) & (2**64 - 1) for k in range(4)] for v in vals], dtype=np.uint64)


@pytest.mark.parametrize("n", [1, 257, 4096])
def test_to_base_and_to_mont_match_integers(pp, O, cuda, n):
    P = pp.ppfr
    x = O.random_fr(n, 0xF00 + n)                      # Montgomery forms
    base = host(P.to_base(dev(x)))
    R_INV = pow(1 << 256, -1, R)
    assert ints(base) == [v * R_INV % R for v in ints(x)]
    assert np.array_equal(host(P.to_mont(dev(base))), x)
    assert ints(base)[:8] == [O.unmont(row) for row in x[:8]]


def test_to_mont_reduces_any_256_bit_input(pp, cuda):
    P = pp.ppfr
    vals = [0, 1, R - 1, R, R + 5, 2 * R + 7, (1 << 256) - 1]
    got = ints(host(P.to_mont(dev(limbs(vals)))))
    assert got == [v * (1 << 256) % R for v in vals]


def test_count_noncanonical(pp, cuda):
    P = pp.ppfr
    vals = [0, R - 1, R, R + 1, (1 << 256) - 1, 12345] * 1000
    assert P.count_noncanonical(dev(limbs(vals))) == 3000
    assert P.count_noncanonical(P.random_fr(1 << 20, 3)) == 0
    assert P.count_noncanonical(P.empty(0)) == 0


def test_raw_file_round_trip(pp, O, cuda, tmp_path):
    P = pp.ppfr
    x = O.random_fr(1000, 77)
    path = str(tmp_path / "in.bin")
    x.tofile(path)
    t = P.read_raw(path)
    assert t.is_pinned() and t.shape == (1000, 4)
    assert np.array_equal(t.numpy().view(np.uint64), x)
    P.write_raw(str(tmp_path / "out.bin"), dev(x))
    assert np.array_equal(np.fromfile(str(tmp_path / "out.bin"), dtype=np.uint64).reshape(-1, 4), x)
    with pytest.raises(ValueError):
        P.read_raw(path, n=1001)


def test_cpp_layer_files_and_conversions(pp, O, cuda, tmp_path):
    n = 513
    x = O.random_fr(n, 99)
    x.tofile(tmp_path / "in.bin")
    r = subprocess.run([DRIVER, "convert", str(n), str(tmp_path / "in.bin"), str(tmp_path)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    base = np.fromfile(tmp_path / "base.bin", dtype=np.uint64).reshape(n, 4)
    R_INV = pow(1 << 256, -1, R)
    assert ints(base) == [v * R_INV % R for v in ints(x)]
    assert np.array_equal(np.fromfile(tmp_path / "mont.bin", dtype=np.uint64).reshape(n, 4), x)
    words = [int(w) for w in open(tmp_path / "base.txt").read().split()]
    assert words == [int(w) for w in base.reshape(-1)]
