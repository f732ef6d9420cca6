"""The C ABI: the library loads without a GPU and exports every entry point
that include/*.h declares (no compute call is made here)."""
from __future__ import annotations

import ctypes
import glob
import os
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(pp_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol(pp):
    L = ctypes.CDLL(os.path.join(ROOT, "ppopp26-artifact_gb300", "libppfr.so"))
    names = declared_symbols()
    assert "pp_ntt" in names and "pp_lde" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_status_strings_and_version(pp):
    L = pp.ppfr.lib()
    assert L.pp_status_string(0) == b"ok"
    assert b"sm_103a" in L.pp_version()


def test_invalid_arguments_are_reported_not_fatal(pp):
    """Argument checks run before any device work, so they hold without a GPU."""
    L = pp.ppfr.lib()
    assert L.pp_ntt(None, None, 10, 0, None) == 1  # PP_E_INVAL
    assert b"aligned" in L.pp_last_error()
    assert L.pp_lde(ctypes.c_void_p(16), ctypes.c_void_p(32), 10, 9, 0, None) == 1  # lambda > 8
    assert L.pp_ntt(ctypes.c_void_p(16), ctypes.c_void_p(16), 31, 0, None) == 5  # unsupported size
    # the integer-rate probe checks its output array before any launch
    L.pp_measure_int_rates_ex.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    out = (ctypes.c_double * 6)()
    assert L.pp_measure_int_rates_ex(None, 6) == 1
    assert L.pp_measure_int_rates_ex(out, 3) == 1
    assert L.pp_measure_int_rates_ex(out, 7) == 1
