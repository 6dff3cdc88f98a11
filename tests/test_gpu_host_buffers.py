"""Host-buffer queries (rmq_query_host / rmq_query_idx_host and their 64-bit
forms): both the direct path (page-locked buffers read and written by the
kernel) and the chunked upload / answer / download pipeline give exactly the
results of the device-buffer calls and of the oracle (GPU)."""
from __future__ import annotations

import numpy as np
import pytest

import rmq_gb300 as R
from conftest import golden_cases, load_golden
from oracle import oracle

pytestmark = pytest.mark.gpu

CHUNK = 1 << 22  # the library's staging chunk


@pytest.mark.parametrize("variant", ["vl", "cl"])
@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.stem)
def test_host_calls_on_golden(cuda, path, variant):
    import torch
    name, a, qs, emin, eidx = load_golden(path)
    dv = torch.from_numpy(a).to(cuda)
    with R.Hierarchy(dv, variant=variant) as h:
        m = h.query_host(qs.astype(np.uint32))
        i, m2 = h.query_idx_host(qs.astype(np.uint32), with_min=True)
        i_only = h.query_idx_host(qs.astype(np.uint32))
    assert m.tobytes() == emin.astype(np.float32).tobytes()
    assert m2.tobytes() == emin.astype(np.float32).tobytes()
    assert np.array_equal(i, eidx.astype(np.uint32))
    assert np.array_equal(i_only, eidx.astype(np.uint32))


def test_host_pipeline_many_chunks_equals_device_call(cuda):
    """More chunks than staging buffers (buffer reuse), a ragged last chunk,
    pageable and page-locked host buffers."""
    import torch
    n = 1 << 22
    a = R.gen_array(n, 7)
    q = 3 * CHUNK + 12345
    qs = R.gen_queries(q, -7, n, 7)
    dv = torch.from_numpy(a).to(cuda)
    with R.Hierarchy(dv, variant="vl") as h:
        dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
        di, dm = h.query_idx(dq, with_min=True)
        torch.cuda.synchronize()
        hi_, hm = h.query_idx_host(qs, with_min=True)  # pageable numpy buffers
        pq = torch.from_numpy(qs.view(np.int32).reshape(-1)).pin_memory()
        pi = torch.empty(q, dtype=torch.int32).pin_memory()
        pm = torch.empty(q, dtype=torch.float32).pin_memory()
        assert h.query_idx_host_raw(int(pq.data_ptr()), q, int(pi.data_ptr()), int(pm.data_ptr())) == R.RMQ_OK
        hmin_only = h.query_host(qs)
    di = di.cpu().numpy().view(np.uint32)
    dm = dm.cpu().numpy()
    assert np.array_equal(hi_, di)
    assert hm.tobytes() == dm.tobytes()
    assert np.array_equal(pi.numpy().view(np.uint32), di)
    assert pm.numpy().tobytes() == dm.tobytes()
    assert hmin_only.tobytes() == dm.tobytes()
    samp = R.sample_indices(q, 1 << 12, 3).astype(np.int64)
    assert np.array_equal(hi_[samp], oracle.rmq_argmin(a, qs[samp]))


def test_host_calls_validate_and_errors(cuda):
    import torch
    a = R.gen_array(5000, 3)
    dv = torch.from_numpy(a).to(cuda)
    qs = np.array([[0, 4999], [10, 9], [7, 5000], [100, 200]], dtype=np.uint32)
    with R.Hierarchy(dv, variant="vl", validate=True) as h:
        with pytest.raises(R.RMQError) as e:
            h.query_idx_host(qs)
        assert e.value.status == R.RMQ_ERR_QUERY_RANGE
        good = h.query_idx_host(qs[[0, 3]])
        assert np.array_equal(good, oracle.rmq_argmin(a, qs[[0, 3]]))
    with R.Hierarchy(dv, variant="vl") as h:
        i, m = h.query_idx_host(qs, with_min=True)  # invalid queries: NaN / all-ones, no status
        assert i[1] == R.NO_POS and i[2] == R.NO_POS and np.isnan(m[1]) and np.isnan(m[2])
        assert h.query_idx_host(qs[:0]).size == 0
        L = R.lib()
        assert L.rmq_query_idx_host(h._h, None, 1, 0x1000, None) == R.RMQ_ERR_ARG
        assert L.rmq_query_idx_host(h._h, qs.ctypes.data, 1, None, None) == R.RMQ_ERR_ARG
        assert L.rmq_query_host(h._h, qs.ctypes.data, 1, None) == R.RMQ_ERR_ARG
        with pytest.raises(R.RMQError) as e:
            h.query_idx_host(qs.astype(np.uint64))  # 64-bit call on a 32-bit handle
        assert e.value.status == R.RMQ_ERR_UNSUPPORTED
    with R.Hierarchy(dv, variant="vl", with_index=False) as h:
        with pytest.raises(R.RMQError) as e:
            h.query_idx_host(qs[[0]])
        assert e.value.status == R.RMQ_ERR_NO_INDEX
        assert h.query_host(qs[[0, 3]]).tobytes() == oracle.rmq_min(a, qs[[0, 3]]).astype(np.float32).tobytes()


@pytest.mark.parametrize("path", golden_cases()[:4], ids=lambda p: p.stem)
def test_host_calls_wide_handle(cuda, path):
    import torch
    name, a, qs, emin, eidx = load_golden(path)
    dv = torch.from_numpy(a).to(cuda)
    with R.Hierarchy(dv, variant="vl", index_bits=64) as h:
        m = h.query_host(qs.astype(np.uint64))
        i, m2 = h.query_idx_host(qs.astype(np.uint64), with_min=True)
        with pytest.raises(R.RMQError) as e:
            h.query_idx_host(qs.astype(np.uint32))
        assert e.value.status == R.RMQ_ERR_UNSUPPORTED
    assert m.tobytes() == emin.astype(np.float32).tobytes()
    assert m2.tobytes() == emin.astype(np.float32).tobytes()
    assert np.array_equal(i, eidx.astype(np.uint64))


def test_page_locked_buffers_direct_path(cuda):
    """Page-locked buffers take the direct path (the kernel reads and writes
    host memory); a misaligned page-locked output falls back to staging; both
    equal the device call, with and without validation."""
    import torch
    n = 1 << 20
    a = R.gen_array(n, 11)
    q = 100003
    qs = R.gen_queries(q, -1, n, 11)
    qs[5] = (9, 3)  # invalid: l > r
    dv = torch.from_numpy(a).to(cuda)
    pq = torch.from_numpy(qs.view(np.int32).reshape(-1)).pin_memory()
    raw = torch.empty(4 * q + 8, dtype=torch.uint8).pin_memory()
    for validate in (False, True):
        with R.Hierarchy(dv, variant="vl", validate=validate) as h:
            dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
            if validate:
                with pytest.raises(R.RMQError):
                    h.query_idx(dq)
                h2 = R.Hierarchy(dv, variant="vl")
                di, dm = h2.query_idx(dq, with_min=True)
                h2.close()
            else:
                di, dm = h.query_idx(dq, with_min=True)
            torch.cuda.synchronize()
            di = di.cpu().numpy().view(np.uint32)
            dm = dm.cpu().numpy()
            pi = torch.empty(q, dtype=torch.int32).pin_memory()
            pm = torch.empty(q, dtype=torch.float32).pin_memory()
            st = h.query_idx_host_raw(int(pq.data_ptr()), q, int(pi.data_ptr()), int(pm.data_ptr()))
            assert st == (R.RMQ_ERR_QUERY_RANGE if validate else R.RMQ_OK)
            assert np.array_equal(pi.numpy().view(np.uint32), di)
            assert pm.numpy().tobytes() == dm.tobytes()
            # misaligned page-locked minima: staged path
            mis = int(raw.data_ptr()) + 2
            st = h.query_idx_host_raw(int(pq.data_ptr()), q, int(pi.data_ptr()), mis)
            assert st == (R.RMQ_ERR_QUERY_RANGE if validate else R.RMQ_OK)
            got = raw.numpy()[2:2 + 4 * q].copy().view(np.float32)
            assert got.tobytes() == dm.tobytes()
            assert np.array_equal(pi.numpy().view(np.uint32), di)


def test_host_calls_from_several_threads_on_one_handle(cuda):
    """Host-buffer calls on one handle from several host threads at once
    (ctypes releases the GIL): the staging pipeline is shared under the
    handle's lock, page-locked buffers take the direct path; every thread
    gets exactly its own queries' results."""
    import threading
    import torch
    n = 1 << 20
    a = R.gen_array(n, 21)
    dv = torch.from_numpy(a).to(cuda)
    sets = [R.gen_queries(150001 + 7 * k, -7 if k % 2 else -1, n, 30 + k) for k in range(4)]
    with R.Hierarchy(dv, variant="vl") as h:
        expect = []
        for qs in sets:
            i, m = h.query_idx(torch.from_numpy(qs.view(np.int32)).to(cuda), with_min=True)
            expect.append((i.cpu().numpy().view(np.uint32), m.cpu().numpy()))
        torch.cuda.synchronize()
        pinned = []
        for qs in sets:
            q = qs.shape[0]
            pinned.append((torch.from_numpy(qs.view(np.int32).reshape(-1)).pin_memory(),
                           torch.empty(q, dtype=torch.int32).pin_memory(),
                           torch.empty(q, dtype=torch.float32).pin_memory()))
        results, errors = {}, []

        def worker(k, direct):
            try:
                for _ in range(3):
                    if direct:
                        pq, pi, pm = pinned[k]
                        st = h.query_idx_host_raw(int(pq.data_ptr()), sets[k].shape[0], int(pi.data_ptr()),
                                                  int(pm.data_ptr()))
                        assert st == R.RMQ_OK
                        got = (pi.numpy().view(np.uint32).copy(), pm.numpy().copy())
                    else:
                        got = h.query_idx_host(sets[k], with_min=True)
                    results[(k, direct)] = got
            except Exception as exc:  # reported to the main thread
                errors.append(exc)

        threads = [threading.Thread(target=worker, args=(k, d)) for k in range(4) for d in (False, True)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    assert not errors, errors
    for (k, direct), (gi, gm) in results.items():
        ei, em = expect[k]
        assert np.array_equal(gi, ei), (k, direct)
        assert gm.tobytes() == em.tobytes(), (k, direct)
    assert len(results) == 8
