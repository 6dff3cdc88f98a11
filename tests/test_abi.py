"""The C ABI library without a GPU: it loads, exports every declared symbol,
plans layouts and rejects bad arguments before touching the device."""
from __future__ import annotations

import ctypes
import re
import subprocess

import pytest

import rmq_gb300 as R
from conftest import ROOT
from oracle import oracle

HEADERS = {
    "rmq_gb300.h": R.LIB_PATH,
    "rmq_gb300_batch.h": R.LIB_PATH,
    "rmq_gb300_serve.h": R.LIB_PATH,
    "rmq_gb300_gen.h": R.GEN_PATH,
}


def declared_functions(header: str) -> list[str]:
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**([a-z][a-z0-9_]*)\s*\(",
                       text, flags=re.M)
    return sorted(set(names))


@pytest.mark.parametrize("header", sorted(HEADERS))
def test_every_declared_symbol_is_exported(header):
    names = declared_functions(header)
    assert len(names) >= 4, names
    so = HEADERS[header]
    out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, f"{so.name} lacks {missing}"
    lib = ctypes.CDLL(str(so))
    for n in names:
        getattr(lib, n)


def test_strerror():
    assert R.strerror(0) == "ok"
    assert "argument" in R.strerror(R.RMQ_ERR_ARG)
    assert R.strerror(12345) == "unknown status"


@pytest.mark.parametrize("variant,rf_log", [("cl", 5), ("vl", 3), ("cl", 3), ("vl", 4), ("auto", 0)])
def test_plan_layout_matches_oracle(variant, rf_log):
    for n in [1, 100, 4096, 1 << 20, 1 << 26, 1 << 28]:
        for t in [64, 1 << 10, 1 << 16]:
            info = R.plan_layout(n, t, rf_log, variant)
            k, sizes, offs = oracle.layout(n, t, info.rf_log)
            assert info.num_levels == k
            assert info.sizes() == sizes
            assert info.offsets() == offs


def test_plan_layout_defaults_and_preconditions():
    cl = R.plan_layout(1 << 20, 0, 0, "cl")
    assert cl.rf_log == 3 and cl.scan_threshold == 64 and cl.lanes == 2  # tuned CL: rf 8, 2 lanes, t 64
    vl = R.plan_layout(1 << 20, 0, 0, "vl")
    assert vl.rf_log == 3 and vl.scan_threshold == 32  # paper's VL: rf 8, t 32
    # the reference's preconditions: t >= 2 rf (CL, src/xxx.h:211), t >= rf (VL, src/xxx.h:938)
    with pytest.raises(R.RMQError) as e:
        R.plan_layout(1 << 20, 63, 5, "cl")
    assert e.value.status == R.RMQ_ERR_ARG
    R.plan_layout(1 << 20, 64, 5, "cl")
    with pytest.raises(R.RMQError):
        R.plan_layout(1 << 20, 7, 3, "vl")
    R.plan_layout(1 << 20, 8, 3, "vl")
    with pytest.raises(R.RMQError):
        R.plan_layout(1 << 20, 64, 6, "vl")
    wide = R.plan_layout(1 << 33, 64, 3, "vl")  # beyond 32-bit indices: a 64-bit layout
    assert wide.index_bits == 64 and wide.sizes()[1] == 1 << 30
    assert R.plan_layout(1 << 20, 64, 3, "vl").index_bits == 32
    with pytest.raises(R.RMQError) as e:
        R.plan_layout((1 << 40) + 1, 64, 3, "vl")
    assert e.value.status == R.RMQ_ERR_UNSUPPORTED


def test_bad_arguments_rejected_before_device_work():
    L = R.lib()
    h = ctypes.c_void_p()
    cfg = R.config()
    assert L.rmq_build(None, 10, ctypes.byref(cfg), None, ctypes.byref(h)) == R.RMQ_ERR_ARG
    assert L.rmq_build(0x1000, 0, ctypes.byref(cfg), None, ctypes.byref(h)) == R.RMQ_ERR_ARG
    assert L.rmq_build(0x1004, 10, ctypes.byref(cfg), None, ctypes.byref(h)) == R.RMQ_ERR_ARG  # misaligned
    assert L.rmq_build(0x1000, 10, ctypes.byref(cfg), None, None) == R.RMQ_ERR_ARG
    bad = R.config(variant=7)
    assert L.rmq_build(0x1000, 10, ctypes.byref(bad), None, ctypes.byref(h)) == R.RMQ_ERR_ARG
    assert L.rmq_query(None, 0x1000, 10, 0x2000, None) == R.RMQ_ERR_ARG
    assert L.rmq_query_idx(None, 0x1000, 10, 0x2000, None, None) == R.RMQ_ERR_ARG
    assert L.rmq_query_host(None, 0x1000, 10, 0x2000) == R.RMQ_ERR_ARG
    assert L.rmq_query_idx_host(None, 0x1000, 10, 0x2000, None) == R.RMQ_ERR_ARG
    assert L.rmq_query64_host(None, 0x1000, 10, 0x2000) == R.RMQ_ERR_ARG
    assert L.rmq_query_idx64_host(None, 0x1000, 10, 0x2000, None) == R.RMQ_ERR_ARG
    assert L.rmq_scan_bruteforce(None, 10, 0x1000, 1, 0x2000, None, None) == R.RMQ_ERR_ARG
    assert L.rmq_scan_bruteforce(0x1000, 10, 0x1004, 1, 0x2000, None, None) == R.RMQ_ERR_ARG
    assert L.rmq_get_info(None, None) == R.RMQ_ERR_ARG
    L.rmq_destroy(None)
    # values, results off their element alignment (checked before any device work)
    assert L.rmq_scan_bruteforce(0x1002, 10, 0x1000, 1, 0x2000, None, None) == R.RMQ_ERR_ARG
    assert L.rmq_scan_bruteforce(0x1000, 10, 0x1000, 1, 0x2002, None, None) == R.RMQ_ERR_ARG
    assert L.rmq_scan_bruteforce(0x1000, 10, 0x1000, 1, None, 0x2001, None) == R.RMQ_ERR_ARG
    static = L.rmq_query_idx_static
    static.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_uint64,
                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    static.restype = ctypes.c_int
    assert static(0x1000, 10, 0, 0x1000, 1, 0x2002, None, None) == R.RMQ_ERR_ARG
    assert static(0x1000, 10, 0, 0x1000, 1, 0x2000, 0x3001, None) == R.RMQ_ERR_ARG
    assert static(0x1010, 10, 0, 0x1000, 1, 0x2000, None, None) == R.RMQ_ERR_ARG


def test_regular_build_has_no_bounds_counter():
    """Only the bounds-checked build counts out-of-level loads."""
    count = ctypes.c_uint64(7)
    assert R.lib().rmq_debug_bounds_violations(ctypes.byref(count)) == R.RMQ_ERR_UNSUPPORTED
    assert count.value == 0
    assert R.lib().rmq_debug_bounds_violations(None) == R.RMQ_ERR_ARG
