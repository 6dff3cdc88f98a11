"""Parity of the CUDA path with the oracle, through the C ABI (GPU only).

Bar: bit-exact fp32 minima and exact uint32 argmin (lowest index on ties),
for every variant / reduction factor / tile width, on the golden fixtures,
on edge cases, and at the workloads' full sizes through sampled oracle checks
plus size-independent properties.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import rmq_gb300 as R
from conftest import golden_cases, load_golden
from oracle import oracle

pytestmark = pytest.mark.gpu

# (variant, rf_log, lanes) configurations exercised everywhere
CONFIGS = [("vl", 3, 0), ("vl-short", 3, 0), ("vl", 4, 0), ("vl", 5, 0),
           ("cl", 5, 8), ("cl", 5, 4), ("cl", 5, 16), ("cl", 5, 32),
           ("cl", 3, 8), ("cl", 4, 16), ("cl", 3, 32), ("cl", 3, 2), ("cl", 4, 2),
           # the reference's ablations of CL (algs 23, 24, 19) as work distributions
           ("cl-noshuffle", 5, 16), ("cl-noshuffle", 3, 2), ("cl-tile", 5, 16), ("cl-tile", 3, 8),
           ("cl-atomic", 5, 16), ("cl-atomic", 3, 2), ("cl-atomic", 4, 32)]
CFG_IDS = [f"{v}-rf{1 << r}-g{g}" for v, r, g in CONFIGS]


def _t_for(variant, rf_log, t=None):
    rf = 1 << rf_log
    if t is not None:
        return max(t, 2 * rf if variant.startswith("cl") else rf)
    return 0


def run(cuda, a, qs, variant, rf_log, lanes, t=None, argmin=True, with_min=True):
    import torch
    dv = torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    dq = torch.from_numpy(np.ascontiguousarray(qs).view(np.int32)).to(cuda)
    with R.Hierarchy(dv, variant=variant, t=_t_for(variant, rf_log, t), rf_log=rf_log, lanes=lanes) as h:
        m = h.query(dq)
        res_min = m.cpu().numpy()
        if argmin:
            i, m2 = h.query_idx(dq, with_min=True)
            res_idx = i.cpu().numpy().view(np.uint32)
            res_min2 = m2.cpu().numpy()
        else:
            res_idx = res_min2 = None
    torch.cuda.synchronize()
    return res_min, res_idx, res_min2


def assert_bits(got, exp, what):
    got = np.asarray(got, dtype=np.float32)
    exp = np.asarray(exp, dtype=np.float32)
    bad = np.flatnonzero(got.view(np.uint32) != exp.view(np.uint32))
    assert bad.size == 0, f"{what}: {bad.size} mismatches, first at {bad[:5]}: got {got[bad[:5]]} expected {exp[bad[:5]]}"


def assert_idx(got, exp, what):
    bad = np.flatnonzero(np.asarray(got, np.uint32) != np.asarray(exp, np.uint32))
    assert bad.size == 0, f"{what}: {bad.size} mismatches, first at {bad[:5]}: got {got[bad[:5]]} expected {exp[bad[:5]]}"


@pytest.mark.parametrize("cfg", CONFIGS, ids=CFG_IDS)
@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.stem)
def test_golden(cuda, path, cfg):
    name, a, qs, emin, eidx = load_golden(path)
    v, r, g = cfg
    for t in (None, 1 << 10):
        m, i, m2 = run(cuda, a, qs, v, r, g, t)
        assert_bits(m, emin, f"{name} min t={t}")
        assert_idx(i, eidx, f"{name} argmin t={t}")
        assert_bits(m2, emin, f"{name} min-with-argmin t={t}")


@pytest.mark.parametrize("cfg", CONFIGS, ids=CFG_IDS)
def test_exhaustive_small(cuda, cfg):
    """Every query of small arrays of awkward sizes, with heavy ties."""
    rng = np.random.default_rng(1)
    v, r, g = cfg
    for n in [1, 2, 3, 7, 8, 9, 31, 33, 64, 100, 257]:
        a = (rng.integers(0, 5, n) / 4).astype(np.float32)
        l, rr = np.triu_indices(n)
        qs = np.stack([l, rr], 1).astype(np.uint32)
        for t in (None, 1, 1 << 20):
            m, i, _ = run(cuda, a, qs, v, r, g, t)
            assert_bits(m, oracle.rmq_min(a, qs), f"n={n} t={t} min")
            assert_idx(i, oracle.rmq_argmin(a, qs), f"n={n} t={t} argmin")


@pytest.mark.parametrize("cfg", CONFIGS, ids=CFG_IDS)
def test_random_sizes_and_thresholds(cuda, cfg):
    rng = np.random.default_rng(2)
    v, r, g = cfg
    for n in [1000, 4099, 65537, 300_001]:
        a = R.gen_array(n, n)
        a[rng.integers(0, n, n // 20)] = a.min()  # ties on the minimum
        q = 20_000
        length = np.minimum(n, np.exp(rng.normal(np.log(max(2, n // 64)), 1.5, q)).astype(np.int64) + 1)
        l = (rng.random(q) * (n - length + 1)).astype(np.int64)
        qs = np.stack([l, l + length - 1], 1).astype(np.uint32)
        for t in (None, 1 << 10, 1 << 16):
            m, i, m2 = run(cuda, a, qs, v, r, g, t)
            assert_bits(m, oracle.rmq_min(a, qs, 8), f"n={n} t={t}")
            assert_idx(i, oracle.rmq_argmin(a, qs, 8), f"n={n} t={t}")
            assert_bits(m2, m, f"n={n} t={t} min pair")


@pytest.mark.parametrize("cfg", CONFIGS, ids=CFG_IDS)
def test_special_values(cuda, cfg):
    """Signed zeros, +inf runs, negatives: bits of the first occurrence."""
    v, r, g = cfg
    n = 5000
    rng = np.random.default_rng(3)
    cases = {
        "all_equal": np.full(n, 0.5, np.float32),
        "all_inf": np.full(n, np.inf, np.float32),
        "zeros_mixed": np.where(rng.random(n) < 0.5, -0.0, 0.0).astype(np.float32),
        # sparse zeros among positives: +0.0 before -0.0, -0.0 before +0.0, one sign only
        "zeros_plus_first": np.where(np.arange(n) % 97 == 5, np.where(np.arange(n) < n // 2, 0.0, -0.0),
                                     1.0 + rng.random(n)).astype(np.float32),
        "zeros_minus_first": np.where(np.arange(n) % 97 == 5, np.where(np.arange(n) < n // 2, -0.0, 0.0),
                                      1.0 + rng.random(n)).astype(np.float32),
        "zeros_plus_only": np.where(np.arange(n) % 211 == 7, 0.0, 1.0 + rng.random(n)).astype(np.float32),
        "zeros_minus_only": np.where(np.arange(n) % 211 == 7, -0.0, 1.0 + rng.random(n)).astype(np.float32),
        "neg": (-rng.random(n)).astype(np.float32),
        "descending": np.arange(n, 0, -1).astype(np.float32),
    }
    l = rng.integers(0, n, 3000)
    rr = np.minimum(n - 1, l + rng.integers(0, 2000, 3000))
    qs = np.stack([l, rr], 1).astype(np.uint32)
    for name, a in cases.items():
        m, i, m2 = run(cuda, a, qs, v, r, g, 64)
        assert_bits(m, oracle.rmq_min(a, qs), name)
        assert_idx(i, oracle.rmq_argmin(a, qs), name)
        assert_bits(m2, oracle.rmq_min(a, qs), name + " pair")


def test_invalid_queries_and_validate(cuda):
    import torch
    n = 1000
    a = R.gen_array(n, 1)
    qs = np.array([[0, 999], [5, 4], [0, 1000], [999, 999], [0xFFFFFFFF, 0xFFFFFFFF]], np.uint32)
    dv = torch.from_numpy(a).to(cuda)
    dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
    for v in ("cl", "vl"):
        with R.Hierarchy(dv, variant=v) as h:
            m = h.query(dq).cpu().numpy()
            i = h.query_idx(dq).cpu().numpy().view(np.uint32)
        assert m[0] == a.min() and np.isnan(m[1]) and np.isnan(m[2]) and m[3] == a[999] and np.isnan(m[4])
        assert i[0] == np.argmin(a) and i[1] == R.NO_POS and i[2] == R.NO_POS and i[3] == 999
        with R.Hierarchy(dv, variant=v, validate=True) as h:
            with pytest.raises(R.RMQError) as e:
                h.query(dq)
            assert e.value.status == R.RMQ_ERR_QUERY_RANGE
            h.query(dq[:1])  # valid subset passes
            with pytest.raises(R.RMQError):
                h.query_idx(dq)


def test_argument_errors(cuda):
    import torch
    a = torch.zeros(1024, device=cuda)
    with pytest.raises(R.RMQError) as e:
        R.Hierarchy(a[1:], variant="vl")  # 4-byte offset breaks 32-byte alignment
    assert e.value.status == R.RMQ_ERR_ARG
    with pytest.raises(R.RMQError):
        R.Hierarchy(a, variant="cl", t=32, rf_log=5)  # t < 2 rf
    with R.Hierarchy(a, variant="vl", with_index=False) as h:
        q = torch.zeros(4, dtype=torch.int32, device=cuda)
        h.query(q)
        with pytest.raises(R.RMQError) as e:
            h.query_idx(q)
        assert e.value.status == R.RMQ_ERR_NO_INDEX
        assert h.query_raw(int(q.data_ptr()) + 4, 1, int(a.data_ptr())) == R.RMQ_ERR_ARG
        assert h.query_raw(int(q.data_ptr()), 0, int(a.data_ptr())) == R.RMQ_OK
    # result pointers off their element alignment are refused before any launch
    with R.Hierarchy(a, variant="vl") as h:
        q = torch.zeros(4, dtype=torch.int32, device=cuda)
        out = torch.zeros(16, dtype=torch.int32, device=cuda)
        base = int(out.data_ptr())
        assert h.query_raw(int(q.data_ptr()), 1, base + 2) == R.RMQ_ERR_ARG
        assert h.query_idx_raw(int(q.data_ptr()), 1, base + 1, base + 16) == R.RMQ_ERR_ARG
        assert h.query_idx_raw(int(q.data_ptr()), 1, base, base + 18) == R.RMQ_ERR_ARG
        assert h.query_idx_raw(int(q.data_ptr()), 1, base, base + 16) == R.RMQ_OK
        torch.cuda.synchronize()


def test_bruteforce_checker_matches_oracle(cuda):
    import torch
    for path in golden_cases():
        name, a, qs, emin, eidx = load_golden(path)
        dv = torch.from_numpy(a).to(cuda)
        dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
        m, i = R.bruteforce(dv, dq)
        assert_bits(m.cpu().numpy(), emin, name)
        assert_idx(i.cpu().numpy().view(np.uint32), eidx, name)


def test_concurrent_streams_same_handle(cuda):
    """A built handle is immutable: queries on several streams at once agree."""
    import torch
    n = 1 << 20
    a = R.gen_array(n, 5)
    qs = R.gen_queries(1 << 16, -1, n, 5)
    dv = torch.from_numpy(a).to(cuda)
    dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
    exp = oracle.Sparse(a).query(qs, 8)
    with R.Hierarchy(dv, variant="vl") as h:
        streams = [torch.cuda.Stream() for _ in range(4)]
        outs = []
        torch.cuda.synchronize()
        for s in streams:
            with torch.cuda.stream(s):
                outs.append(h.query_idx(dq, with_min=True, stream=s))
        torch.cuda.synchronize()
    for i, m in outs:
        assert_bits(m.cpu().numpy(), exp[0], "min")
        assert_idx(i.cpu().numpy().view(np.uint32), exp[1], "argmin")


# ---- full-size workloads ----------------------------------------------------

def _full_check(cuda, a, qs, sample_seed, cfgs, ts):
    """Full-size check: every query against the GPU brute-force checker where
    affordable, a seeded sample against the CPU sparse oracle, and
    size-independent properties (A[argmin] == min, l <= argmin <= r, all
    configurations agree) on all queries."""
    import torch
    dv = torch.from_numpy(a).to(cuda)
    dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
    q = qs.shape[0]
    samp = R.sample_indices(q, 1 << 15, sample_seed).astype(np.int64)
    sm, si = oracle.Sparse(a).query(qs[samp], 0)
    ref_m = ref_i = None
    for v, r, g in cfgs:
        for t in ts:
            with R.Hierarchy(dv, variant=v, t=_t_for(v, r, t), rf_log=r, lanes=g) as h:
                m = h.query(dq)
                i, m2 = h.query_idx(dq, with_min=True)
            mm = m.cpu().numpy()
            ii = i.cpu().numpy().view(np.uint32)
            assert_bits(mm[samp], sm, f"{v} rf{1 << r} t={t} sample min")
            assert_idx(ii[samp], si, f"{v} rf{1 << r} t={t} sample argmin")
            assert torch.equal(m, m2)
            if ref_m is None:
                ref_m, ref_i = m, i
                ii64 = ii.astype(np.int64)
                assert ((ii64 >= qs[:, 0]) & (ii64 <= qs[:, 1])).all()
                assert_bits(a[ii], mm, "A[argmin] == min")
            else:
                assert torch.equal(m, ref_m) and torch.equal(i, ref_i), f"{v} rf{1 << r} t={t} disagrees"
            del m, i, m2
    return dv, dq, ref_m, ref_i


def test_full_size_medium_lognormal(cuda):
    """n = 2^26, q = 2^26, lognormal lengths (median 2^13, sigma 1): every
    query against the GPU brute-force checker, plus the sampled oracle."""
    import torch
    n = q = 1 << 26
    a = R.gen_array(n, 42)
    qs = R.gen_queries(q, -7, n, 42)
    cfgs = [("vl", 3, 0), ("cl", 5, 8), ("vl", 4, 0)]
    dv, dq, m, i = _full_check(cuda, a, qs, 42, cfgs, [1 << 10, 1 << 16])
    bm, bi = R.bruteforce(dv, dq)
    torch.cuda.synchronize()
    assert torch.equal(bm.view(torch.int32), m.view(torch.int32)), "min vs brute force"
    assert torch.equal(bi, i), "argmin vs brute force"


def test_full_size_large_mixed_ties(cuda):
    """n = 2^28 with 1% of entries set to the global minimum, q = 2^27 with the
    three-way length mixture; argmin (ties to the lowest index)."""
    n = 1 << 28
    q = 1 << 27
    a = R.gen_array(n, 7)
    R.plant_min_ties(a, 0.01, 7)
    qs = R.gen_queries(q, -8, n, 7)
    _full_check(cuda, a, qs, 7, [("vl", 3, 0), ("cl", 5, 8)], [1 << 10])


@pytest.mark.parametrize("n", [1025 * 8192, 1025 * 8192 + 5, 3 * (1 << 22) + 13, (1 << 24) + 8191])
def test_streamed_build_sizes(cuda, n):
    """Arrays of more than 1024 tiles of 8192 entries, where the fused build
    kernel leaves the levels above its tiles to the tail and step kernels,
    some with a partial last tile: every tile's block minima, heavy ties and
    signed zeros, with queries spanning each tile, crossing each tile boundary
    and of random lengths, against the GPU brute-force checker, for every
    reduction factor and both variants at their smallest t (every level is
    read)."""
    import torch
    rng = np.random.default_rng(n)
    a = rng.integers(-50, 50, n).astype(np.float32)
    a[rng.random(n) < 0.02] = -0.0
    a[rng.random(n) < 0.01] = 0.0
    tiles = (n + 8191) // 8192
    starts = np.arange(tiles, dtype=np.int64) * 8192
    whole = np.stack([starts, np.minimum(starts + 8191, n - 1)], 1)
    cross = np.stack([np.maximum(starts[1:] - 37, 0), np.minimum(starts[1:] + 100, n - 1)], 1)
    l = rng.integers(0, n, 1 << 18)
    ln = np.exp(rng.uniform(0, np.log(1 << 20), l.size)).astype(np.int64)
    rnd = np.stack([l, np.minimum(l + ln, n - 1)], 1)
    qs = np.concatenate([whole, cross, rnd]).astype(np.uint32)
    dv = torch.from_numpy(a).to(cuda)
    dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
    bm, bi = R.bruteforce(dv, dq)
    for v, r, g in [("vl", 3, 0), ("vl", 4, 0), ("vl", 5, 0), ("cl", 3, 2), ("cl", 5, 8)]:
        with R.Hierarchy(dv, variant=v, t=_t_for(v, r, 1), rf_log=r, lanes=g) as h:
            i, m = h.query_idx(dq, with_min=True)
            m1 = h.query(dq)
        torch.cuda.synchronize()
        assert torch.equal(m.view(torch.int32), bm.view(torch.int32)), f"{v} rf{1 << r} min"
        assert torch.equal(m1.view(torch.int32), bm.view(torch.int32)), f"{v} rf{1 << r} min-only"
        assert torch.equal(i, bi), f"{v} rf{1 << r} argmin"
    # the same array under a 64-bit handle (64-bit positions in every level)
    with R.Hierarchy(dv, variant="vl", t=8, rf_log=3, index_bits=64) as h:
        i64, m64 = h.query_idx64(torch.from_numpy(qs.astype(np.int64)).to(cuda), with_min=True)
    torch.cuda.synchronize()
    assert torch.equal(m64.view(torch.int32), bm.view(torch.int32)), "64-bit min"
    assert torch.equal(i64, bi.to(torch.int64)), "64-bit argmin"


def test_cl_ablations_preconditions_and_info(cuda):
    """The ablated CL work distributions keep CL's precondition t >= 2 rf and
    report their variant; the atomic combine takes thresholds below 2^27."""
    import torch
    a = torch.zeros(1 << 12, dtype=torch.float32, device=cuda)
    for v, code in (("cl-noshuffle", 3), ("cl-tile", 4), ("cl-atomic", 5)):
        with pytest.raises(R.RMQError) as e:
            R.Hierarchy(a, variant=v, t=31, rf_log=4)  # t < 2 rf
        assert e.value.status == R.RMQ_ERR_ARG
        with R.Hierarchy(a, variant=v, t=64, rf_log=4, lanes=4) as h:
            info = h.info()
            assert info.variant == code and info.lanes == 4 and info.rf_log == 4
    with pytest.raises(R.RMQError) as e:
        R.Hierarchy(a, variant="cl-atomic", t=1 << 27, rf_log=3)
    assert e.value.status == R.RMQ_ERR_UNSUPPORTED
