"""The oracle against the reference: golden fixtures, the reference build, and
the fast sparse-table oracle against brute force (CPU only)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle import oracle


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.stem)
def test_bruteforce_oracle_matches_golden(path):
    name, a, qs, emin, eidx = load_golden(path)
    got_min = oracle.rmq_min(a, qs, 4)
    got_idx = oracle.rmq_argmin(a, qs, 4)
    assert got_min.tobytes() == emin.astype(np.float32).tobytes(), name
    assert np.array_equal(got_idx, eidx.astype(np.uint32)), name


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.stem)
def test_sparse_oracle_matches_golden(path):
    name, a, qs, emin, eidx = load_golden(path)
    m, i = oracle.Sparse(a).query(qs, 4)
    assert m.tobytes() == emin.astype(np.float32).tobytes(), name
    assert np.array_equal(i, eidx.astype(np.uint32)), name


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_sparse_matches_bruteforce_random(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 200_000))
    # few distinct values -> many ties
    a = rng.integers(0, 17, n).astype(np.float32) / 4.0
    q = 4000
    l = rng.integers(0, n, q)
    r = np.minimum(n - 1, l + rng.integers(0, max(1, n // int(rng.integers(1, 50))), q))
    qs = np.stack([l, r], 1).astype(np.uint32)
    m, i = oracle.Sparse(a).query(qs, 4)
    assert m.tobytes() == oracle.rmq_min(a, qs, 4).tobytes()
    assert np.array_equal(i, oracle.rmq_argmin(a, qs, 4))


def test_invalid_queries_marked():
    a = np.arange(10, dtype=np.float32)
    qs = np.array([[3, 2], [0, 10], [9, 9]], dtype=np.uint32)
    m = oracle.rmq_min(a, qs)
    i = oracle.rmq_argmin(a, qs)
    assert np.isnan(m[0]) and np.isnan(m[1]) and m[2] == 9
    assert i[0] == 0xFFFFFFFF and i[1] == 0xFFFFFFFF and i[2] == 9


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not built here")
@pytest.mark.parametrize("seed", [5, 27722, 833241])
def test_oracle_matches_reference_build(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1000, 300_000))
    a = oracle.ref_array(n, seed)
    a[rng.integers(0, n, n // 50)] = a.min()  # planted ties
    qs = oracle.ref_queries(3000, -6, n, seed)
    assert oracle.rmq_min(a, qs, 4).tobytes() == oracle.ref_min(a, qs).tobytes()
    assert np.array_equal(oracle.rmq_argmin(a, qs, 4), oracle.ref_argmin(a, qs))


def _reference_layout_rule(n, t, rf_log):
    """Line-by-line reading of src/xxx.h:225-243 (host loop)."""
    num_levels, size, off = 1, n, 0
    sizes, offs = [n], [(1 << 64) - 1]
    while True:
        if num_levels >= 20 or size <= t:
            break
        size = (size + (1 << rf_log) - 1) >> rf_log
        off = (off + 31) & ~31
        offs.append(off)
        sizes.append(size)
        num_levels += 1
        off += size
    return num_levels, sizes, offs


@pytest.mark.parametrize("rf_log", [2, 3, 4, 5])
def test_layout_restatement(rf_log):
    for n in [1, 2, 31, 32, 33, 1000, 4096, 65537, 1 << 20, (1 << 26) + 5, 1 << 28, 0xFFFFFF00]:
        for t in [1, 8, 32, 64, 1 << 10, 1 << 16, 1 << 30]:
            assert oracle.layout(n, t, rf_log) == _reference_layout_rule(n, t, rf_log)
