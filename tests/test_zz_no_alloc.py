"""rmq_query_idx_static: range argmin without any device allocation.

Callers that cannot allocate device memory when they query (hosts that keep
the whole device in their own memory pool, latency-bound callers that must
not call cudaMalloc / cudaFree because those can block and synchronise the
device) use this entry point: the hierarchy lives in a fixed 8 MiB array the
library holds on each device, the caller passes only inputs and outputs.

Checked through the C ABI against the handle-based rmq_query_idx, bit for
bit, on two calls in a row (a larger array first, so stale coarse levels
from the first call would show up in the second).  This file is collected
last so that a stopping run has already run every other test.
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
