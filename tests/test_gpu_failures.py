"""Failure paths on the device side, made on the host (GPU): allocation
failures reported as RMQ_ERR_OOM with nothing left behind, HBM-budget
exhaustion in the server, a poisoned request among healthy ones, a batch
whose launch fails (injected on the host) and a bounded wait that gives up.  Nothing here faults, traps or hangs the GPU:
every allocation that fails does so before any kernel could touch the
(deliberately small) input buffers."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import rmq_gb300 as R
from oracle import oracle

pytestmark = pytest.mark.gpu


def _queries(rng, n, q):
    length = np.minimum(n, np.exp(rng.normal(np.log(64.0), 2.0, q)).astype(np.int64) + 1)
    lo = (rng.random(q) * (n - length + 1)).astype(np.int64)
    return np.stack([lo, lo + length - 1], 1).astype(np.uint32)


def test_build_allocation_failure_reports_oom_and_context_stays_usable(cuda):
    import torch
    small = torch.zeros(1024, dtype=torch.float32, device=cuda)
    # 2^40 entries (64-bit handle): the level buffer alone would need ~1.9 TB,
    # so rmq_build's first allocation fails before any kernel runs.
    cfg = R.config("vl", 0, 0, 0, True, False, False, 64)
    h = ctypes.c_void_p()
    st = R.lib().rmq_build(ctypes.c_void_p(small.data_ptr()), 1 << 40, ctypes.byref(cfg), None, ctypes.byref(h))
    assert st == R.RMQ_ERR_OOM and not h.value
    # the context is healthy: a normal build and query still work
    a = R.gen_array(1 << 16, 5)
    rng = np.random.default_rng(5)
    qs = _queries(rng, a.size, 4096)
    with R.Hierarchy(torch.from_numpy(a).to(cuda)) as hh:
        got = hh.query_idx(torch.from_numpy(qs.view(np.int32)).to(cuda)).cpu().numpy().view(np.uint32)
    assert np.array_equal(got, oracle.rmq_argmin(a, qs))


def test_batch_allocation_failure_reports_oom(cuda):
    import torch
    small = torch.zeros(1024, dtype=torch.float32, device=cuda)
    num = 4096
    sizes = np.full(num, 0xFFFFFF00, dtype=np.uint64)  # ~10 TB of levels: cannot be allocated
    offs = (np.arange(num, dtype=np.uint64) << np.uint64(32))
    with pytest.raises(R.RMQError) as e:
        R.Batch(small, offs, sizes)
    assert e.value.status == R.RMQ_ERR_OOM


def test_server_create_beyond_device_memory(cuda):
    with pytest.raises(R.RMQError) as e:
        R.Server(hbm_budget_bytes=1 << 41)  # 2 TiB arena
    assert e.value.status == R.RMQ_ERR_OOM


def test_server_budget_exhaustion_and_recovery(cuda):
    rng = np.random.default_rng(8)
    with R.Server(hbm_budget_bytes=16 << 20, slots=2) as srv:
        with pytest.raises(R.RMQError) as e:
            srv.register_generated(1 << 23, 1)  # 32 MiB of values alone
        assert e.value.status == R.RMQ_ERR_OOM
        big = np.zeros(1 << 23, np.float32)
        with pytest.raises(R.RMQError) as e:
            srv.register_host(big)
        assert e.value.status == R.RMQ_ERR_OOM
        a = rng.random(5000).astype(np.float32)
        aid = srv.register_host(a)
        qs = _queries(rng, a.size, 3000)
        oi = np.empty(qs.shape[0], np.uint32)
        st, _ = srv.wait(srv.submit(aid, qs, oi, None))
        assert st == R.RMQ_OK
        assert np.array_equal(oi, oracle.rmq_argmin(a, qs))


def test_server_poisoned_request_leaves_the_others_intact(cuda):
    rng = np.random.default_rng(9)
    a = rng.random(1 << 16).astype(np.float32)
    with R.Server(hbm_budget_bytes=64 << 20, slots=2) as srv:
        aid = srv.register_host(a)
        good1 = _queries(rng, a.size, 5000)
        bad = _queries(rng, a.size, 5000)
        bad[17] = (100, 50)          # l > r
        bad[4000] = (0, a.size)      # r = n
        good2 = _queries(rng, a.size, 5000)
        outs = [(np.empty(5000, np.uint32), np.empty(5000, np.float32)) for _ in range(3)]
        rids = [srv.submit(aid, qs, oi, om) for qs, (oi, om) in zip((good1, bad, good2), outs)]
        sts = [srv.wait(r)[0] for r in rids]
    assert sts == [R.RMQ_OK, R.RMQ_ERR_QUERY_RANGE, R.RMQ_OK]
    for qs, (oi, om), poisoned in zip((good1, bad, good2), outs, (False, True, False)):
        keep = np.ones(qs.shape[0], bool)
        if poisoned:
            keep[[17, 4000]] = False
            assert oi[17] == R.NO_POS and oi[4000] == R.NO_POS and np.isnan(om[17]) and np.isnan(om[4000])
        assert np.array_equal(oi[keep], oracle.rmq_argmin(a, qs[keep]))
        assert om[keep].tobytes() == oracle.rmq_min(a, qs[keep]).tobytes()


def test_server_wait_gives_up_then_completes(cuda):
    rng = np.random.default_rng(10)
    a = rng.random(1 << 20).astype(np.float32)
    with R.Server(hbm_budget_bytes=64 << 20) as srv:
        aid = srv.register_host(a)
        qs = _queries(rng, a.size, 1 << 20)
        oi = np.empty(qs.shape[0], np.uint32)
        rid = srv.submit(aid, qs, oi, None)
        st, _ = srv.wait(rid, timeout_ms=0)  # not done the moment it was submitted
        assert st == R.RMQ_ERR_TIMEOUT
        st, lat = srv.wait(rid)
        assert st == R.RMQ_OK and lat > 0
    samp = np.arange(0, qs.shape[0], 97)
    assert np.array_equal(oi[samp], oracle.rmq_argmin(a, qs[samp]))


def test_server_failed_batch_reports_cuda_error_to_its_waiter(cuda):
    """A batch whose launch fails completes its requests with RMQ_ERR_CUDA
    (argmin all ones, minima NaN), the status set together with completion so
    a waiter woken at once sees it; the server then keeps serving."""
    rng = np.random.default_rng(11)
    a = rng.random(1 << 16).astype(np.float32)
    with R.Server(hbm_budget_bytes=64 << 20, slots=2) as srv:
        aid = srv.register_host(a)
        qs = _queries(rng, a.size, 4000)
        warm = np.empty(qs.shape[0], np.uint32)
        assert srv.wait(srv.submit(aid, qs, warm, None))[0] == R.RMQ_OK  # array built
        srv.fail_next_batches(1)
        oi = np.zeros(qs.shape[0], np.uint32)
        om = np.zeros(qs.shape[0], np.float32)
        st, _ = srv.wait(srv.submit(aid, qs, oi, om))
        assert st == R.RMQ_ERR_CUDA
        assert np.all(oi == R.NO_POS) and np.all(np.isnan(om))
        for _ in range(3):  # the failed batch left nothing behind
            oi2 = np.empty(qs.shape[0], np.uint32)
            om2 = np.empty(qs.shape[0], np.float32)
            st, _ = srv.wait(srv.submit(aid, qs, oi2, om2))
            assert st == R.RMQ_OK
            assert np.array_equal(oi2, oracle.rmq_argmin(a, qs))
            assert om2.tobytes() == oracle.rmq_min(a, qs).tobytes()
        assert srv.stats()["requests_done"] == 5
