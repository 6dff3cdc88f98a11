"""Shared test setup: marker registration, import paths, fixtures.

Tests marked `gpu` need a CUDA device and call the library through its C ABI
(ctypes); all others run on the CPU: the oracle against the golden fixtures
and the reference build, the host logic, and the C ABI's symbol table.
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "gpu-rmq_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: full-size workload")


def pytest_sessionfinish(session, exitstatus):
    """In a run against the bounds-checked build (RMQ_EXPECT_CHECKED_LIB set,
    RMQ_GB300_LIB naming librmq_gb300_checked.so): after the tests, read the
    device-side count of out-of-level loads and fail the run unless it is 0."""
    if not os.environ.get("RMQ_EXPECT_CHECKED_LIB") or exitstatus != 0:
        return
    import ctypes
    import rmq_gb300 as R
    count = ctypes.c_uint64()
    st = R.lib().rmq_debug_bounds_violations(ctypes.byref(count))
    print(f"\nbounds-checked build: status {st}, out-of-level loads {count.value}")
    if st != R.RMQ_OK or count.value != 0:
        session.exitstatus = 3


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the library, generators, driver and oracle once per session."""
    sys.path.insert(0, str(PKG))
    import build  # gpu-rmq_gb300/build.py
    build.build_all()
    yield


def golden_cases():
    return sorted(p for p in GOLDEN.glob("*.npz") if p.name != "sample_indices.npz")


def load_golden(path: Path):
    """Returns (name, array, queries, expected_min, expected_argmin)."""
    import rmq_gb300 as R
    import hashlib
    z = np.load(path)
    if str(z["kind"]) == "generated":
        a = R.gen_array(int(z["n"]), int(z["array_seed"]))
        assert hashlib.sha256(a.tobytes()).hexdigest() == str(z["array_sha256"]), \
            f"{path.name}: generated array differs from the reference generator's"
    else:
        a = np.array(z["array"], dtype=np.float32)
    return path.stem, a, np.array(z["queries"], dtype=np.uint32), np.array(z["expected_min"]), \
        np.array(z["expected_argmin"])


@pytest.fixture(scope="session")
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device in this environment")
    return torch.device("cuda:0")
