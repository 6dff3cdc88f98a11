"""The query server (GPU): results identical alone and in the mix and equal
to the oracle; coalescing into shared batches; eviction and re-admission
under a small HBM budget; invalid queries reported per request."""
from __future__ import annotations

import numpy as np
import pytest

import rmq_gb300 as R
from oracle import oracle

pytestmark = pytest.mark.gpu


def _queries(rng, n, q):
    length = np.minimum(n, np.exp(rng.normal(np.log(max(2.0, n / 50)), 1.2, q)).astype(np.int64) + 1)
    l = (rng.random(q) * (n - length + 1)).astype(np.int64)
    return np.ascontiguousarray(np.stack([l, l + length - 1], 1).astype(np.uint32))


def test_same_alone_and_in_mix(cuda):
    rng = np.random.default_rng(5)
    sizes = [1, 7, 100, 4099, 65_537, 1 << 20, 300_001, 8192, 77, 1 << 18]
    arrays = []
    for n in sizes:
        a = (rng.integers(0, 40, n) / 3).astype(np.float32)  # ties
        arrays.append(a)
    reqs = []
    for i in range(80):
        aid = int(rng.integers(0, len(sizes)))
        reqs.append((aid, _queries(rng, sizes[aid], int(rng.integers(1, 5000)))))
    with R.Server(hbm_budget_bytes=1 << 30, slots=4) as srv:
        ids = [srv.register_host(a) for a in arrays]
        assert ids == list(range(len(sizes)))
        alone = []
        for aid, qs in reqs:
            oi = np.empty(qs.shape[0], np.uint32)
            om = np.empty(qs.shape[0], np.float32)
            st, lat = srv.wait(srv.submit(aid, qs, oi, om))
            assert st == R.RMQ_OK and lat > 0
            alone.append((oi, om))
        mix = []
        rids = []
        for aid, qs in reqs:
            oi = np.empty(qs.shape[0], np.uint32)
            om = np.empty(qs.shape[0], np.float32)
            rids.append(srv.submit(aid, qs, oi, om))
            mix.append((oi, om))
        srv.drain()
        for rid in rids:
            assert srv.wait(rid)[0] == R.RMQ_OK
        stats = srv.stats()
    assert stats["max_requests_per_batch"] > 1  # the mix was coalesced
    for (aid, qs), (ai, am), (mi, mm) in zip(reqs, alone, mix):
        assert np.array_equal(ai, mi) and ai.tobytes() == mi.tobytes()
        assert am.tobytes() == mm.tobytes()
        assert np.array_equal(ai, oracle.rmq_argmin(arrays[aid], qs))
        assert am.tobytes() == oracle.rmq_min(arrays[aid], qs).tobytes()


def test_eviction_and_readmission(cuda):
    import torch
    rng = np.random.default_rng(6)
    n = 1 << 20  # 4 MiB of values + levels per array
    seeds = [11, 12, 13, 14, 15, 16]
    with R.Server(hbm_budget_bytes=16 << 20, slots=2) as srv:  # room for ~3 arrays
        ids = [srv.register_generated(n, s) for s in seeds]
        expected = {}
        for aid, seed in zip(ids, seeds):
            v = torch.empty(n, dtype=torch.float32, device=cuda)
            R.gen_values_device(v, seed)
            torch.cuda.synchronize()
            expected[aid] = v.cpu().numpy()
        for rnd in range(3):
            for aid in ids:
                qs = _queries(rng, n, 2000)
                oi = np.empty(qs.shape[0], np.uint32)
                om = np.empty(qs.shape[0], np.float32)
                st, _ = srv.wait(srv.submit(aid, qs, oi, om))
                assert st == R.RMQ_OK
                assert np.array_equal(oi, oracle.rmq_argmin(expected[aid], qs))
                assert om.tobytes() == oracle.rmq_min(expected[aid], qs).tobytes()
        stats = srv.stats()
    assert stats["evictions"] > 0 and stats["readmissions"] > 0
    assert stats["resident_bytes"] <= 16 << 20


def test_invalid_query_and_replay(cuda):
    rng = np.random.default_rng(7)
    a = rng.random(1000).astype(np.float32)
    with R.Server(hbm_budget_bytes=64 << 20) as srv:
        aid = srv.register_host(a)
        qs = np.array([[0, 999], [10, 5], [0, 1000]], dtype=np.uint32)
        oi = np.empty(3, np.uint32)
        om = np.empty(3, np.float32)
        rid = srv.submit(aid, qs, oi, om)
        st, _ = srv.wait(rid)
        assert st == R.RMQ_ERR_QUERY_RANGE
        assert oi[0] == np.argmin(a) and oi[1] == R.NO_POS and oi[2] == R.NO_POS and np.isnan(om[1])
        assert srv.wait(rid)[0] == R.RMQ_ERR_ARG  # collected by the first wait
        # a small replayed stream: a registration and requests before and after it
        lr = _queries(rng, 1000, 3000)
        ev = np.zeros(4, dtype=R.TRACE_DTYPE)
        ev["t_arrival_s"] = [0.0, 0.001, 0.002, 0.003]
        ev["kind"] = [0, 1, 0, 0]
        ev["array_id"] = [aid, 0, aid, 1]
        ev["n"] = [0, 1000, 0, 0]
        ev["seed"] = [0, 3, 0, 0]
        ev["q_offset"] = [0, 0, 1000, 2000]
        ev["q"] = [1000, 0, 1000, 1000]
        out_i = np.empty(3000, np.uint32)
        out_m = np.empty(3000, np.float32)
        lat, wall = srv.replay(ev, lr, out_i, out_m)
        assert lat[1] == -1 and (lat[[0, 2, 3]] > 0).all() and wall > 0
        assert np.array_equal(out_i[:2000], oracle.rmq_argmin(a, lr[:2000]))


def test_serial_loop_comparator_matches_oracle(cuda):
    """rmq_serve_serial_loop (the server's per-request comparator) answers
    every query request of a trace exactly, from page-locked and from
    ordinary host buffers."""
    import torch
    rng = np.random.default_rng(12)
    sizes = [5000, 1 << 16, 70_001]
    arrays = [rng.random(n).astype(np.float32) for n in sizes]
    hs = [R.Hierarchy(torch.from_numpy(a).to(cuda), variant="vl", t=64) for a in arrays]
    ev = np.zeros(12, dtype=R.TRACE_DTYPE)
    parts, off = [], 0
    for i in range(ev.size):
        if i == 5:
            ev["kind"][i] = 1  # a registration: skipped by the loop
            continue
        aid = int(rng.integers(0, len(sizes)))
        qs = _queries(rng, sizes[aid], int(rng.integers(1, 3000)))
        ev["array_id"][i], ev["q_offset"][i], ev["q"][i] = aid, off, qs.shape[0]
        parts.append(qs)
        off += qs.shape[0]
    lr = np.ascontiguousarray(np.concatenate(parts))
    for pinned in (True, False):
        if pinned:
            h_lr = torch.from_numpy(lr.view(np.int32).reshape(-1)).pin_memory()
            oi = torch.zeros(off, dtype=torch.int32).pin_memory()
            om = torch.zeros(off, dtype=torch.float32).pin_memory()
        else:
            h_lr, oi, om = lr, np.zeros(off, np.uint32), np.zeros(off, np.float32)
        wall = R.serve_serial_loop(hs, ev, h_lr, oi, om)
        assert wall > 0
        gi = oi.numpy().view(np.uint32) if pinned else oi
        gm = om.numpy() if pinned else om
        for i in range(ev.size):
            if ev["kind"][i] != 0:
                continue
            o, q, aid = int(ev["q_offset"][i]), int(ev["q"][i]), int(ev["array_id"][i])
            assert np.array_equal(gi[o:o + q], oracle.rmq_argmin(arrays[aid], lr[o:o + q]))
            assert gm[o:o + q].tobytes() == oracle.rmq_min(arrays[aid], lr[o:o + q]).tobytes()
    for h in hs:
        h.close()


def test_page_locked_requests_are_answered_in_place(cuda):
    """Requests whose buffers are page-locked are read and written in place by
    the batch kernel (no staging); mixed in one batch with staged requests,
    every result equals the oracle's, minima-only and argmin-only requests
    included, and invalid queries are reported per request."""
    import torch
    rng = np.random.default_rng(13)
    sizes = [3000, 1 << 17, 70_001]
    arrays = [(rng.integers(0, 60, n) / 9).astype(np.float32) for n in sizes]  # ties
    with R.Server(hbm_budget_bytes=256 << 20, slots=3) as srv:
        ids = [srv.register_host(a) for a in arrays]
        for aid in ids:  # every array built before the mix
            w = np.zeros((1, 2), np.uint32)
            assert srv.wait(srv.submit(aid, w, np.empty(1, np.uint32), None))[0] == R.RMQ_OK
        prepared = []
        for i in range(60):
            aid = int(rng.integers(0, len(sizes)))
            qs = _queries(rng, sizes[aid], int(rng.integers(1, 4000)))
            pinned = i % 3 != 0
            bad = i % 11 == 5
            if bad:
                qs[0] = (7, 3)  # l > r
            if pinned:
                t_q = torch.from_numpy(qs.view(np.int32).reshape(-1)).pin_memory()
                lr = t_q.numpy().view(np.uint32).reshape(-1, 2)
                oi_t = torch.zeros(qs.shape[0], dtype=torch.int32).pin_memory()
                om_t = torch.zeros(qs.shape[0], dtype=torch.float32).pin_memory()
                keep = (t_q, oi_t, om_t)
                oi = oi_t.numpy().view(np.uint32)
                om = om_t.numpy()
            else:
                lr, oi, om, keep = qs, np.zeros(qs.shape[0], np.uint32), np.zeros(qs.shape[0], np.float32), None
            which = i % 4  # 0: both outputs, 1: argmin only, 2: minima only, 3: both
            prepared.append((aid, qs, lr, oi, om, which, bad, keep, pinned))
        # all buffers ready first: the submissions then arrive close together
        reqs = [(srv.submit(aid, lr, oi if which != 2 else None, om if which != 1 else None),
                 aid, qs, oi, om, which, bad, keep)
                for aid, qs, lr, oi, om, which, bad, keep, _ in prepared]
        for rid, aid, qs, oi, om, which, bad, keep in reqs:
            st, _ = srv.wait(rid)
            assert st == (R.RMQ_ERR_QUERY_RANGE if bad else R.RMQ_OK)
            ok = np.ones(qs.shape[0], bool)
            if bad:
                ok[0] = False
                if which != 2:
                    assert oi[0] == R.NO_POS
                if which != 1:
                    assert np.isnan(om[0])
            if which != 2:
                assert np.array_equal(oi[ok], oracle.rmq_argmin(arrays[aid], qs[ok]))
            if which != 1:
                assert om[ok].tobytes() == oracle.rmq_min(arrays[aid], qs[ok]).tobytes()
        stats = srv.stats()
    # exactly the requests with page-locked buffers were answered in place
    assert stats["direct_requests"] == sum(1 for x in prepared if x[-1])


def test_concurrent_submitters_and_registration(cuda):
    """Several host threads submit to and wait on one server at once (each
    waiting on its own requests while the others' are in flight) while
    another thread registers arrays: every request's results equal the
    oracle and every request completes."""
    import threading
    rng = np.random.default_rng(9)
    sizes = [5000, 1 << 16, 123457, 1 << 19]
    arrays = [(rng.integers(0, 50, n) / 7).astype(np.float32) for n in sizes]
    errors, done = [], []
    with R.Server(hbm_budget_bytes=1 << 30, slots=4) as srv:
        ids = [srv.register_host(a) for a in arrays]

        def check(pending):
            for rid, aid, qs, oi, om in pending:
                st, _ = srv.wait(rid)
                assert st == R.RMQ_OK
                assert np.array_equal(oi, oracle.rmq_argmin(arrays[aid], qs))
                assert om.tobytes() == oracle.rmq_min(arrays[aid], qs).tobytes()
                done.append(rid)

        def submitter(k):
            try:
                r = np.random.default_rng(100 + k)
                pending = []
                for j in range(40):
                    aid = int(r.integers(0, len(sizes)))
                    qs = _queries(r, sizes[aid], int(r.integers(1, 3000)))
                    oi = np.empty(qs.shape[0], np.uint32)
                    om = np.empty(qs.shape[0], np.float32)
                    pending.append((srv.submit(ids[aid], qs, oi, om), aid, qs, oi, om))
                    if j % 5 == 4:
                        check(pending)
                        pending = []
                check(pending)
            except Exception as exc:  # reported to the main thread
                errors.append(exc)

        def registrar():
            try:
                for s in range(6):
                    srv.register_generated(1 << 16, 500 + s)
            except Exception as exc:
                errors.append(exc)

        threads = [threading.Thread(target=submitter, args=(k,)) for k in range(4)]
        threads.append(threading.Thread(target=registrar))
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        stats = srv.stats()
    assert not errors, errors
    assert len(done) == 4 * 40 and len(set(done)) == 4 * 40
    assert stats["registrations"] == len(sizes) + 6
