"""rmq_query_idx_static: range argmin without any device allocation.

Callers that cannot allocate device memory when they query (hosts that keep
the whole device in their own memory pool, latency-bound callers that must
not call cudaMalloc / cudaFree because those can block and synchronise the
device) use this entry point: the hierarchy lives in a fixed 8 MiB array the
library holds on each device, the caller passes only inputs and outputs.

Checked through the C ABI against the handle-based rmq_query_idx, bit for
bit, on two calls in a row (a larger array first, so stale coarse levels
from the first call would show up in the second), with a non-default scan
threshold, with no queries, and with invalid queries; and that a call leaves
the device's free memory unchanged.  This file is collected last so that a
stopping run has already run every other test.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import rmq_gb300 as R

pytestmark = pytest.mark.gpu

_P = ctypes.c_void_p
_U64 = ctypes.c_uint64


def _entry():
    f = R.lib().rmq_query_idx_static
    f.argtypes = [_P, _U64, _U64, _P, _U64, _P, _P, _P]
    f.restype = ctypes.c_int
    return f


def test_static_matches_handle_queries_two_calls(cuda):
    import torch
    f = _entry()
    stream = torch.cuda.current_stream().cuda_stream
    for n, q, seed in [(1 << 22, 1 << 18, 11), (100_003, 50_000, 12)]:
        a = R.gen_array(n, seed)
        a[::1001] = a.min()  # ties on the minimum
        qs = R.gen_queries(q, -6, n, seed)
        dv = torch.from_numpy(a).to(cuda)
        dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
        with R.Hierarchy(dv, variant="vl", t=32, rf_log=3) as h:
            exp_i, exp_m = h.query_idx(dq, with_min=True)
        got_i = torch.full((q,), -1, dtype=torch.int32, device=cuda)
        got_m = torch.full((q,), -1.0, dtype=torch.float32, device=cuda)
        st = f(dv.data_ptr(), n, 0, dq.data_ptr(), q, got_i.data_ptr(), got_m.data_ptr(), stream)
        assert st == R.RMQ_OK, R.strerror(st)
        torch.cuda.synchronize()
        assert torch.equal(got_i, exp_i), f"argmin differs (n={n})"
        assert torch.equal(got_m.view(torch.int32), exp_m.view(torch.int32)), f"minima differ (n={n})"


def test_static_rejects_sizes_beyond_the_limit(cuda):
    import torch
    f = _entry()
    n = (1 << 22) + 1
    dv = torch.zeros(n, dtype=torch.float32, device=cuda)
    dq = torch.zeros(2, dtype=torch.int32, device=cuda)
    out = torch.empty(1, dtype=torch.int32, device=cuda)
    st = f(dv.data_ptr(), n, 0, dq.data_ptr(), 1, out.data_ptr(), None, None)
    assert st == R.RMQ_ERR_UNSUPPORTED


def _handle_results(cuda, dv, dq, t):
    with R.Hierarchy(dv, variant="vl", t=t, rf_log=3) as h:
        return h.query_idx(dq, with_min=True)


def test_static_other_threshold_empty_and_invalid_queries(cuda):
    import torch
    f = _entry()
    n, q = 1 << 20, 1 << 16
    a = R.gen_array(n, 21)
    qs = R.gen_queries(q, -1, n, 21)
    qs[5] = (100, 50)        # l > r
    qs[q - 1] = (0, n)       # r = n
    dv = torch.from_numpy(a).to(cuda)
    dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
    exp_i, exp_m = _handle_results(cuda, dv, dq, 8)
    got_i = torch.zeros(q, dtype=torch.int32, device=cuda)
    got_m = torch.zeros(q, dtype=torch.float32, device=cuda)
    st = f(dv.data_ptr(), n, 8, dq.data_ptr(), q, got_i.data_ptr(), got_m.data_ptr(), None)
    assert st == R.RMQ_OK, R.strerror(st)
    torch.cuda.synchronize()
    assert torch.equal(got_i, exp_i) and torch.equal(got_m.view(torch.int32), exp_m.view(torch.int32))
    gi = got_i.cpu().numpy().view(np.uint32)
    gm = got_m.cpu().numpy()
    assert gi[5] == R.NO_POS and gi[q - 1] == R.NO_POS and np.isnan(gm[5]) and np.isnan(gm[q - 1])
    keep = np.ones(q, bool)
    keep[[5, q - 1]] = False
    from oracle import oracle
    assert np.array_equal(gi[keep], oracle.rmq_argmin(a, qs[keep]))
    # no queries: nothing is written
    sentinel = torch.full((4,), 7, dtype=torch.int32, device=cuda)
    assert f(dv.data_ptr(), n, 0, None, 0, sentinel.data_ptr(), None, None) == R.RMQ_OK
    torch.cuda.synchronize()
    assert torch.equal(sentinel, torch.full((4,), 7, dtype=torch.int32, device=cuda))


def test_static_call_leaves_free_device_memory_unchanged(cuda):
    import torch
    f = _entry()
    n, q = 1 << 22, 1 << 18
    a = R.gen_array(n, 31)
    qs = R.gen_queries(q, -6, n, 31)
    dv = torch.from_numpy(a).to(cuda)
    dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
    oi = torch.empty(q, dtype=torch.int32, device=cuda)
    om = torch.empty(q, dtype=torch.float32, device=cuda)
    # The first call on a device may load the array and the kernels; after it,
    # a call must not change the free memory.
    assert f(dv.data_ptr(), n, 0, dq.data_ptr(), q, oi.data_ptr(), om.data_ptr(), None) == R.RMQ_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(cuda)
    for _ in range(3):
        assert f(dv.data_ptr(), n, 0, dq.data_ptr(), q, oi.data_ptr(), om.data_ptr(), None) == R.RMQ_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(cuda)
    assert free1 == free0
