"""Shared fixtures.  CPU tests run anywhere; tests marked ``gpu`` need a GB300
(or any sm_103a device) and the compiled library."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device and the compiled library")


@pytest.fixture(scope="session")
def O():
    """The CPU oracle (test infrastructure)."""
    from oracle import oracle

    oracle.lib()
    return oracle


@pytest.fixture(scope="session")
def pp():
    """The product package, loaded through its C ABI; builds it if needed."""
    import __graft_entry__ as ge

    if not os.path.exists(os.path.join(ge.PKG_DIR, "libppfr.so")):
        ge._load_build_module().build()
    return ge.load_package()


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    torch.cuda.set_device(0)
    return torch


def host(t) -> np.ndarray:
    """Device tensor (n, 4) int64 -> numpy uint64 (n, 4)."""
    return t.detach().cpu().numpy().view(np.uint64).reshape(-1, 4)


def dev(a: np.ndarray):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint64).view(np.int64)).cuda()


@pytest.fixture(scope="session")
def golden():
    d = os.path.join(ROOT, "tests", "golden")
    import json

    with open(os.path.join(d, "ntt_tables.json")) as f:
        tables = json.load(f)
    arrays = dict(np.load(os.path.join(d, "reference_cpu.npz")))
    return tables, arrays


def table_elem(hexlimbs) -> np.ndarray:
    return np.array([int(h, 16) for h in hexlimbs], dtype=np.uint64)
