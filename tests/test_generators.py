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
