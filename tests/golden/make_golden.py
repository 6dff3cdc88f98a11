"""Writes tests/golden/*.npz from the reference's own code (oracle/_ref).

Run where the reference sources are present (after the build):
    python tests/golden/make_golden.py

Each fixture holds the inputs (or, for generated arrays, the generator
arguments plus a SHA-256 of the reference-generated array), the queries, and
the reference's cpu_rmq / cpu_rmq_idx outputs (src/cpu_methods.h:18-77).
"""
from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent

# (name, n, array seed, lr, q, query seed, trivial)
GENERATED = [
    ("uniform_n4096", 4096, 42, -1, 1024, 42, False),
    ("lognormal_medium_n65536", 65536, 7, -2, 1024, 7, False),
    ("lognormal_small_n1000", 1000, 11, -3, 1024, 11, False),
    ("lognormal_n256_n65536", 65536, 5, -4, 512, 5, False),
    ("mixed_n100003", 100003, 913, -6, 2048, 913, False),
    ("constant64_trivial_n5000", 5000, 3, 64, 4096, 3, True),
    ("constant1_n777", 777, 27722, 1, 512, 27722, False),
    ("uniform_n1", 1, 1, -1, 16, 1, False),
]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def special_array(n: int, seed: int) -> np.ndarray:
    """Tie-heavy array with signed zeros, +inf and negatives."""
    rng = np.random.default_rng(seed)
    pool = np.array([0.5, 0.25, np.inf, -0.0, 0.0, -1.0, 3.0, -1.0, 0.25, np.inf], dtype=np.float32)
    a = pool[rng.integers(0, pool.size, n)]
    a[: n // 10] = np.inf  # a run of +inf at the start
    a[n // 2: n // 2 + 64] = -0.0  # a run of negative zeros
    a[n // 2 + 64: n // 2 + 128] = 0.0
    return a.astype(np.float32)


def special_queries(n: int, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    qs = [(0, 0), (0, n - 1), (n - 1, n - 1), (n // 2, n // 2 + 127), (n // 2 + 64, n // 2 + 127),
          (0, n // 10 - 1), (0, n // 10), (n // 2 - 1, n // 2 + 200)]
    for length in [1, 2, 7, 8, 9, 15, 16, 17, 31, 32, 33, 63, 64, 65, 127, 128, 129, 255, 256, 257,
                   511, 512, 513, 1023, 1024, 1025, 2047, 2049, 4095, 4097]:
        if length > n:
            continue
        for _ in range(8):
            l = int(rng.integers(0, n - length + 1))
            qs.append((l, l + length - 1))
    for _ in range(512):
        l = int(rng.integers(0, n))
        r = int(rng.integers(l, n))
        qs.append((l, r))
    return np.array(qs, dtype=np.uint32)


def main() -> None:
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/librmq_ref.so not built (reference sources absent?)")
    for name, n, aseed, lr, q, qseed, trivial in GENERATED:
        a = oracle.ref_array(n, aseed)
        qs = oracle.ref_queries(q, lr, n, qseed, trivial)
        np.savez_compressed(
            OUT / f"{name}.npz", kind="generated", n=n, array_seed=aseed, array_sha256=sha(a),
            lr=lr, q=q, query_seed=qseed, trivial=int(trivial), queries=qs,
            expected_min=oracle.ref_min(a, qs), expected_argmin=oracle.ref_argmin(a, qs))
    for name, n, seed in [("special_n3000", 3000, 1), ("special_n4099", 4099, 2)]:
        a = special_array(n, seed)
        qs = special_queries(n, seed)
        np.savez_compressed(OUT / f"{name}.npz", kind="explicit", n=n, array=a, queries=qs,
                            expected_min=oracle.ref_min(a, qs), expected_argmin=oracle.ref_argmin(a, qs))
    # reference sampling used by --randTrivialCheck (src/rand.cuh:219-240)
    np.savez_compressed(OUT / "sample_indices.npz", original=1 << 20, sample=1 << 12, seed=42,
                        indices=oracle.ref_sample_indices(1 << 20, 1 << 12, 42))
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()
