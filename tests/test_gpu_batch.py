"""Batched build/query over many arrays, and the device generators (GPU).

Every query of every array must equal the oracle bit for bit, whatever the
path: separate build + query launches, the captured graph (twice), and after
autotuning (which rebuilds with the chosen threshold)."""
from __future__ import annotations

import numpy as np
import pytest

import rmq_gb300 as R
from oracle import oracle

pytestmark = pytest.mark.gpu


def _make_batch(cuda, sizes, seed):
    import torch
    rng = np.random.default_rng(seed)
    offs, total = R.pack_offsets(sizes)
    host = np.full(total, np.nan, dtype=np.float32)  # padding must never be read as data
    arrays = []
    for a, n in enumerate(sizes):
        x = (rng.integers(0, 50, n) / 7).astype(np.float32)  # many ties
        if n > 3:
            x[rng.integers(0, n, max(1, n // 100))] = x.min()
        host[int(offs[a]): int(offs[a]) + n] = x
        arrays.append(x)
    qcounts = [int(rng.integers(0, 3 * n + 5)) if a % 7 else 0 for a, n in enumerate(sizes)]
    qo = np.zeros(len(sizes) + 1, dtype=np.uint64)
    qo[1:] = np.cumsum(qcounts)
    qs = np.zeros((int(qo[-1]), 2), dtype=np.uint32)
    for a, n in enumerate(sizes):
        c = qcounts[a]
        if c == 0:
            continue
        length = np.minimum(n, np.exp(rng.normal(np.log(max(1.0, np.sqrt(n))), 1.0, c)).astype(np.int64) + 1)
        l = (rng.random(c) * (n - length + 1)).astype(np.int64)
        qs[int(qo[a]): int(qo[a + 1])] = np.stack([l, l + length - 1], 1)
    dv = torch.from_numpy(host).to(cuda)
    dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
    return dv, dq, offs, arrays, qs, qo


def _expected(arrays, qs, qo):
    emin = np.empty(qs.shape[0], np.float32)
    eidx = np.empty(qs.shape[0], np.uint32)
    for a, x in enumerate(arrays):
        s, e = int(qo[a]), int(qo[a + 1])
        if e > s:
            emin[s:e] = oracle.rmq_min(x, qs[s:e])
            eidx[s:e] = oracle.rmq_argmin(x, qs[s:e])
    return emin, eidx


def _check(out_min, out_idx, emin, eidx, what):
    m = out_min.cpu().numpy()
    i = out_idx.cpu().numpy().view(np.uint32)
    bad = np.flatnonzero(m.view(np.uint32) != emin.view(np.uint32))
    assert bad.size == 0, f"{what}: {bad.size} minima differ, first {bad[:5]}"
    bad = np.flatnonzero(i != eidx)
    assert bad.size == 0, f"{what}: {bad.size} argmin differ, first {bad[:5]}"


@pytest.mark.parametrize("seed", [0, 1])
def test_batch_matches_oracle(cuda, seed):
    import torch
    rng = np.random.default_rng(100 + seed)
    sizes = [1, 2, 7, 8, 9, 63, 64, 65, 8191, 8192, 8193, 100_003] + \
            [int(x) for x in np.exp(rng.uniform(np.log(1 << 10), np.log(1 << 20), 60))]
    dv, dq, offs, arrays, qs, qo = _make_batch(cuda, sizes, seed)
    emin, eidx = _expected(arrays, qs, qo)
    q = qs.shape[0]
    out_min = torch.empty(q, dtype=torch.float32, device=cuda)
    out_idx = torch.empty(q, dtype=torch.int32, device=cuda)
    with R.Batch(dv, offs, sizes, t=64) as b:
        b.set_queries(dq, qo, out_idx, out_min)
        b.build()
        b.query()
        torch.cuda.synchronize()
        _check(out_min, out_idx, emin, eidx, "build+query")
        for rep in range(2):
            out_min.fill_(-1)
            out_idx.fill_(-1)
            b.run()
            torch.cuda.synchronize()
            _check(out_min, out_idx, emin, eidx, f"graph run {rep}")
        info = b.autotune()
        assert info.scan_threshold in (16, 32, 64, 256, 1024) and info.query_block in (64, 128, 256, 512)
        out_min.fill_(-1)
        out_idx.fill_(-1)
        b.run()
        torch.cuda.synchronize()
        _check(out_min, out_idx, emin, eidx, "after autotune")
        # minima only
        only = torch.full((q,), -1.0, dtype=torch.float32, device=cuda)
        b.set_queries(dq, qo, None, only)
        b.query()
        torch.cuda.synchronize()
        assert np.array_equal(only.cpu().numpy().view(np.uint32), emin.view(np.uint32))


def test_batch_argument_errors(cuda):
    import torch
    dv = torch.zeros(64, device=cuda)
    with pytest.raises(R.RMQError):
        R.Batch(dv, [0, 4], [4, 4])  # offset 4 is not 32-byte aligned
    with pytest.raises(R.RMQError):
        R.Batch(dv, [0], [0])  # empty array
    with R.Batch(dv, [0, 8], [8, 8], with_index=False) as b:
        dq = torch.zeros(4, dtype=torch.int32, device=cuda)
        out = torch.empty(2, dtype=torch.int32, device=cuda)
        with pytest.raises(R.RMQError) as e:
            b.set_queries(dq, [0, 1, 2], out, None)
        assert e.value.status == R.RMQ_ERR_NO_INDEX
        with pytest.raises(R.RMQError):
            b.run()  # no queries registered
    with R.Batch(dv, [0, 8], [8, 8]) as b:
        dq = torch.zeros(4, dtype=torch.int32, device=cuda)
        out = torch.empty(4, dtype=torch.int32, device=cuda)
        qo = np.array([0, 1, 2], dtype=np.uint64)
        set_q = R._bind_batch().rmq_batch_set_queries
        # result pointers off their 4-byte alignment are refused
        assert set_q(b._h, dq.data_ptr(), qo.ctypes.data, out.data_ptr() + 2, None, None) == R.RMQ_ERR_ARG
        assert set_q(b._h, dq.data_ptr(), qo.ctypes.data, out.data_ptr(), out.data_ptr() + 9,
                     None) == R.RMQ_ERR_ARG


def test_device_generators(cuda):
    import torch
    v = torch.empty(1 << 20, dtype=torch.float32, device=cuda)
    R.gen_values_device(v, 7)
    x = v.cpu().numpy()
    assert x.min() >= 0.0 and x.max() < 1.0 and abs(x.mean() - 0.5) < 0.01
    v2 = torch.empty_like(v)
    R.gen_values_device(v2, 7)
    assert torch.equal(v, v2)
    n = 1 << 20
    for law, med, sig in [(0, 1.0, 0.0), (1, 8192.0, 1.0), (1, 32.0, 0.7)]:
        qd = torch.empty((1 << 18, 2), dtype=torch.int32, device=cuda)
        R.gen_queries_device(qd, n, law, med, sig, 3)
        qh = qd.cpu().numpy().view(np.uint32).astype(np.int64)
        length = qh[:, 1] - qh[:, 0] + 1
        assert (qh[:, 0] <= qh[:, 1]).all() and (qh[:, 1] < n).all()
        if law == 1:
            assert 0.8 * med < np.median(length) < 1.25 * med
        else:
            assert abs(np.mean(length) / n - 0.5) < 0.01


def test_tuning_cache_and_set_tuning(cuda, tmp_path):
    """A tuning choice stored in the JSON cache is applied (no tuning pass)
    on the same workload and gives the same exact results; set_tuning checks
    its arguments and the level capacity."""
    import json
    import torch
    rng = np.random.default_rng(5)
    sizes = [int(x) for x in np.exp(rng.uniform(np.log(1 << 10), np.log(1 << 18), 40))]
    dv, dq, offs, arrays, qs, qo = _make_batch(cuda, sizes, 5)
    emin, eidx = _expected(arrays, qs, qo)
    q = qs.shape[0]
    cache = tmp_path / "tuning.json"
    out_min = torch.empty(q, dtype=torch.float32, device=cuda)
    out_idx = torch.empty(q, dtype=torch.int32, device=cuda)
    with R.Batch(dv, offs, sizes, t=64) as b:
        b.set_queries(dq, qo, out_idx, out_min)
        first = b.autotune(cache=cache)
        table = json.loads(cache.read_text())
        assert list(table.values())[0]["scan_threshold"] == first.scan_threshold
        key = b.workload_key()
    # pretend an earlier run chose (t = 1024, 256 threads): the cache is applied as is
    table[key] = {"scan_threshold": 1024, "query_block": 256, "query_ms": 1.0, "arrays": len(sizes)}
    cache.write_text(json.dumps(table))
    with R.Batch(dv, offs, sizes, t=64) as b:
        b.set_queries(dq, qo, out_idx, out_min)
        info = b.autotune(cache=cache)
        assert info.scan_threshold == 1024 and info.query_block == 256
        out_min.fill_(-1)
        out_idx.fill_(-1)
        b.run()
        torch.cuda.synchronize()
        _check(out_min, out_idx, emin, eidx, "cached tuning")
        for bad_t, bad_block in ((4, 128), (64, 48), (64, 1024)):
            with pytest.raises(R.RMQError) as e:
                b.set_tuning(bad_t, bad_block)
            assert e.value.status == R.RMQ_ERR_ARG
        with pytest.raises(R.RMQError) as e:
            b.set_tuning(8, 128)  # deeper than the levels allocated for t >= 16
        assert e.value.status == R.RMQ_ERR_UNSUPPORTED
        b.set_tuning(32, 512)
        b.run()
        torch.cuda.synchronize()
        _check(out_min, out_idx, emin, eidx, "set_tuning(32, 512)")


def test_per_array_loop_matches_batched(cuda):
    """rmq_batch_run_per_array (the per-array loop of the plain build and
    query kernels over the batch's buffers) gives the batched results, which
    are the oracle's."""
    import torch
    rng = np.random.default_rng(9)
    sizes = [1, 8, 9, 8193, 100_003] + [int(x) for x in np.exp(rng.uniform(np.log(1 << 10), np.log(1 << 19), 30))]
    dv, dq, offs, arrays, qs, qo = _make_batch(cuda, sizes, 9)
    emin, eidx = _expected(arrays, qs, qo)
    q = qs.shape[0]
    out_min = torch.empty(q, dtype=torch.float32, device=cuda)
    out_idx = torch.empty(q, dtype=torch.int32, device=cuda)
    with R.Batch(dv, offs, sizes, t=32) as b:
        b.set_queries(dq, qo, out_idx, out_min)
        for rep in range(2):
            out_min.fill_(-1)
            out_idx.fill_(-1)
            b.run_per_array()
            torch.cuda.synchronize()
            _check(out_min, out_idx, emin, eidx, f"per-array loop {rep}")
        b.run()
        torch.cuda.synchronize()
        _check(out_min, out_idx, emin, eidx, "graph after the loop")


def test_class_thresholds(cuda):
    """One scan threshold per array-size class: any combination gives exact
    results, and the autotuner reports a valid choice per class."""
    import torch
    rng = np.random.default_rng(21)
    sizes = [int(x) for x in np.exp(rng.uniform(np.log(1 << 10), np.log(1 << 20), 30))] + [100, 20_000, 300_000]
    dv, dq, offs, arrays, qs, qo = _make_batch(cuda, sizes, 21)
    emin, eidx = _expected(arrays, qs, qo)
    q = qs.shape[0]
    out_min = torch.empty(q, dtype=torch.float32, device=cuda)
    out_idx = torch.empty(q, dtype=torch.int32, device=cuda)
    with R.Batch(dv, offs, sizes, t=64) as b:
        b.set_queries(dq, qo, out_idx, out_min)
        for tc in ([16, 256, 1024], [1024, 16, 32], [64, 64, 16]):
            b.set_class_tuning(tc, 128)
            info = b.info()
            assert list(info.class_threshold) == tc and info.scan_threshold == tc[2]
            out_min.fill_(-1)
            out_idx.fill_(-1)
            b.run()
            torch.cuda.synchronize()
            _check(out_min, out_idx, emin, eidx, f"class thresholds {tc}")
            out_min.fill_(-1)
            out_idx.fill_(-1)
            b.run_per_array()
            torch.cuda.synchronize()
            _check(out_min, out_idx, emin, eidx, f"per-array loop, class thresholds {tc}")
        with pytest.raises(R.RMQError):
            b.set_class_tuning([4, 64, 64], 128)
        info = b.autotune()
        assert all(t in (16, 32, 64, 256, 1024) for t in info.class_threshold)
        assert list(info.class_upper)[:2] == [1 << 14, 1 << 18]
        out_min.fill_(-1)
        out_idx.fill_(-1)
        b.run()
        torch.cuda.synchronize()
        _check(out_min, out_idx, emin, eidx, "after the per-class autotune")
