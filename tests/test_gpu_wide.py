"""64-bit handles: the reference's IS_LONG path (uint64 indices, ulong2
queries) for arrays beyond 2^32 entries (GPU)."""
from __future__ import annotations

import numpy as np
import pytest

import rmq_gb300 as R
from conftest import golden_cases, load_golden
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.stem)
def test_wide_handle_on_golden(cuda, path):
    import torch
    name, a, qs, emin, eidx = load_golden(path)
    dv = torch.from_numpy(a).to(cuda)
    dq = torch.from_numpy(qs.astype(np.int64)).to(cuda)
    with R.Hierarchy(dv, variant="vl", index_bits=64) as h:
        assert h.info().index_bits == 64
        m = h.query64(dq)
        i, m2 = h.query_idx64(dq, with_min=True)
        with pytest.raises(R.RMQError) as e:
            h.query(torch.from_numpy(qs.view(np.int32)).to(cuda))
        assert e.value.status == R.RMQ_ERR_UNSUPPORTED
    assert m.cpu().numpy().tobytes() == emin.astype(np.float32).tobytes()
    assert m2.cpu().numpy().tobytes() == emin.astype(np.float32).tobytes()
    assert np.array_equal(i.cpu().numpy(), eidx.astype(np.int64))


def test_wide_rejects_cl_and_narrow_calls(cuda):
    import torch
    dv = torch.zeros(1024, device=cuda)
    with pytest.raises(R.RMQError) as e:
        R.Hierarchy(dv, variant="cl", index_bits=64)
    assert e.value.status == R.RMQ_ERR_UNSUPPORTED
    with R.Hierarchy(dv, variant="vl") as h:
        with pytest.raises(R.RMQError) as e:
            h.query64(torch.zeros((1, 2), dtype=torch.int64, device=cuda))
        assert e.value.status == R.RMQ_ERR_UNSUPPORTED


def test_beyond_2_pow_32_entries(cuda):
    """n = 2^32 + 2^25 + 8 device-generated values (16 GiB): queries in a window
    across the 2^32 boundary equal those of a 32-bit handle on that window
    (shifted), and full-range queries equal torch's first-occurrence argmin."""
    import torch
    n = (1 << 32) + (1 << 25) + 8
    v = torch.empty(n, dtype=torch.float32, device=cuda)
    R.gen_values_device(v, 2024)
    w0, wn = (1 << 32) - (1 << 25), 1 << 26  # window across the boundary (32-byte aligned)
    assert w0 + wn <= n
    rng = np.random.default_rng(9)
    q = 1 << 18
    length = np.minimum(wn, np.exp(rng.normal(np.log(8192.0), 2.0, q)).astype(np.int64) + 1)
    l = (rng.random(q) * (wn - length + 1)).astype(np.int64)
    local = np.stack([l, l + length - 1], 1)
    with R.Hierarchy(v, variant="vl", t=64) as hw:
        assert hw.info().index_bits == 64
        dq = torch.from_numpy(local + w0).to(cuda)
        wi, wm = hw.query_idx64(dq, with_min=True)
        with R.Hierarchy(v[w0:w0 + wn], variant="vl", t=64) as hn:
            ni, nm = hn.query_idx(torch.from_numpy(local.astype(np.uint32).view(np.int32)).to(cuda), with_min=True)
        torch.cuda.synchronize()
        assert not bool(torch.isnan(wm).any()) and int((wi < 0).sum()) == 0  # every query valid
        assert torch.equal(wm.view(torch.int32), nm.view(torch.int32))
        assert torch.equal(wi, ni.to(torch.int64) + w0)
        full = torch.tensor([[0, n - 1], [12345, n - 1], [(1 << 32) - 5, (1 << 32) + 5], [1, (1 << 32) + 1000]],
                            dtype=torch.int64, device=cuda)
        fi, fm = hw.query_idx64(full, with_min=True)
        torch.cuda.synchronize()
        for k in range(full.shape[0]):
            lo, hi = int(full[k, 0]), int(full[k, 1])
            seg = v[lo:hi + 1]
            ai = int(torch.argmin(seg)) + lo  # first occurrence of the minimum
            assert int(fi[k]) == ai, (lo, hi, int(fi[k]), ai)
            assert fm[k].view(torch.int32) == v[ai].view(torch.int32)
