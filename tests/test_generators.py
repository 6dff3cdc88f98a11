"""The product's input generators against the reference's (CPU only)."""
from __future__ import annotations

import numpy as np
import pytest

import rmq_gb300 as R
from conftest import GOLDEN, golden_cases
from oracle import oracle


@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.stem)
def test_generated_fixture_queries(path):
    z = np.load(path)
    if str(z["kind"]) != "generated":
        pytest.skip("explicit fixture")
    qs = R.gen_queries(int(z["q"]), int(z["lr"]), int(z["n"]), int(z["query_seed"]), bool(z["trivial"]))
    assert np.array_equal(qs, z["queries"])


def test_sample_indices_fixture():
    z = np.load(GOLDEN / "sample_indices.npz")
    got = R.sample_indices(int(z["original"]), int(z["sample"]), int(z["seed"]))
    assert np.array_equal(got, z["indices"])
    assert np.array_equal(R.sample_indices(10, 20, 1), np.arange(10, dtype=np.uint32))


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not built here")
@pytest.mark.parametrize("lr", [1, 5, 100, -1, -2, -3, -4, -5, -6])
@pytest.mark.parametrize("n,seed", [(1 << 16, 1), (12345, 913), (1 << 22, 27722)])
def test_generators_match_reference_build(lr, n, seed):
    if lr > n:
        pytest.skip("length above n")
    assert R.gen_array(n, seed).tobytes() == oracle.ref_array(n, seed).tobytes()
    for trivial in (False, True):
        assert np.array_equal(R.gen_queries(5000, lr, n, seed, trivial),
                              oracle.ref_queries(5000, lr, n, seed, trivial))


@pytest.mark.parametrize("lr", [-7, -8])
def test_new_length_laws(lr):
    n = 1 << 20
    qs = R.gen_queries(200_000, lr, n, 4)
    l = qs[:, 0].astype(np.int64)
    r = qs[:, 1].astype(np.int64)
    length = r - l + 1
    assert (l >= 0).all() and (r < n).all() and (length >= 1).all()
    assert np.array_equal(qs, R.gen_queries(200_000, lr, n, 4))  # deterministic
    assert not np.array_equal(qs, R.gen_queries(200_000, lr, n, 5))  # seeded
    if lr == -7:
        med = np.median(length)
        assert 7000 < med < 9500, med  # median 2^13
        assert 0.9 < np.std(np.log(length)) < 1.1  # sigma 1 (slight clamp effect)
    else:
        # one third each: uniform [1, n], ~2^13 and ~2^5 medians
        assert (length > 200_000).mean() > 0.2
        assert (length < 100).mean() > 0.25


def test_plant_min_ties():
    a = R.gen_array(1 << 16, 3)
    m = a.min()
    R.plant_min_ties(a, 0.01, 9)
    assert (a == m).sum() >= round(0.01 * (1 << 16))
    assert a.min() == m


def test_bad_length_law():
    with pytest.raises(ValueError):
        R.gen_queries(10, -9, 100, 1)
    with pytest.raises(ValueError):
        R.gen_queries(10, 101, 100, 1)


# ---- the oracle's own generators (used by the benchmark's reference arm) -----

@pytest.mark.parametrize("path", golden_cases(), ids=lambda p: p.stem)
def test_oracle_generators_reproduce_fixtures(path):
    """The oracle's restatement of the reference generators against the
    fixtures the reference build wrote (array by SHA-256, queries exactly)."""
    import hashlib
    z = np.load(path)
    if str(z["kind"]) != "generated" or bool(z["trivial"]):
        pytest.skip("explicit or trivial-check fixture")
    a = oracle.gen_array(int(z["n"]), int(z["array_seed"]))
    assert hashlib.sha256(a.tobytes()).hexdigest() == str(z["array_sha256"])
    qs = oracle.gen_queries(int(z["q"]), int(z["lr"]), int(z["n"]), int(z["query_seed"]))
    assert np.array_equal(qs, z["queries"])


@pytest.mark.parametrize("lr", [1, 37, -1, -2, -3, -4, -5, -6, -7, -8])
@pytest.mark.parametrize("n,seed", [(1 << 16, 1), (12345, 913), (1 << 22, 42)])
def test_oracle_generators_equal_product_generators(lr, n, seed):
    """Two independent implementations of one draw order give the same inputs
    (the benchmark's two arms time the same workload)."""
    assert oracle.gen_array(n, seed).tobytes() == R.gen_array(n, seed).tobytes()
    assert np.array_equal(oracle.gen_queries(20_000, lr, n, seed), R.gen_queries(20_000, lr, n, seed))
    a, b = R.gen_array(n, seed), R.gen_array(n, seed)
    assert oracle.plant_min_ties(a, 0.01, seed).tobytes() == R.plant_min_ties(b, 0.01, seed).tobytes()


@pytest.mark.skipif(not oracle.ref_available(), reason="reference sources not built here")
@pytest.mark.parametrize("lr", [1, 100, -1, -2, -3, -4, -5, -6])
def test_oracle_generators_match_reference_build(lr):
    n, seed = 1 << 20, 833241
    assert oracle.gen_array(n, seed).tobytes() == oracle.ref_array(n, seed).tobytes()
    assert np.array_equal(oracle.gen_queries(5000, lr, n, seed), oracle.ref_queries(5000, lr, n, seed, False))


def test_oracle_reference_schedule_scan_equals_checker():
    """cpu_rmq / cpu_rmq_idx as the reference schedules them (the timed CPU
    baseline) give the checker's results."""
    a = R.gen_array(1 << 16, 5)
    qs = R.gen_queries(3000, -6, 1 << 16, 5)
    assert oracle.cpu_rmq(a, qs).tobytes() == oracle.rmq_min(a, qs).tobytes()
    assert np.array_equal(oracle.cpu_rmq_idx(a, qs), oracle.rmq_argmin(a, qs))
