"""Seeded random parity sweep (GPU): sizes around the level, tile and
L1-threshold boundaries, random thresholds down to each variant's minimum,
every work distribution, three length laws, ties and signed zeros.  Every
case must equal the oracle bit for bit (minima from both query calls, and the
argmin)."""
from __future__ import annotations

import numpy as np
import pytest

import rmq_gb300 as R
from oracle import oracle

pytestmark = pytest.mark.gpu

CFGS = [("vl", 3, 0), ("vl-short", 3, 0), ("vl", 4, 0), ("vl", 5, 0), ("cl", 3, 2), ("cl", 4, 4), ("cl", 5, 8), ("cl", 3, 32),
        ("cl", 5, 16), ("cl-noshuffle", 4, 8), ("cl-tile", 3, 4), ("cl-atomic", 5, 16)]
BOUNDARY_SIZES = [1, 2, 7, 8, 9, 15, 16, 17, 63, 64, 65, 511, 512, 513, 4095, 4096, 4097, 8191, 8192, 8193,
                  16383, 16384, 16385, 32768, 131071, 131072, 131073, 1 << 20]


def _case(rng):
    n = int(rng.choice(BOUNDARY_SIZES)) if rng.random() < 0.4 else int(np.exp(rng.uniform(0, np.log(2 << 20))))
    n = max(1, n + int(rng.integers(-3, 4))) if rng.random() < 0.3 else max(1, n)
    kind = int(rng.integers(0, 4))
    if kind == 0:
        a = rng.random(n).astype(np.float32)
    elif kind == 1:
        a = (rng.integers(0, 20, n) / 3).astype(np.float32)  # heavy ties
    elif kind == 2:  # sparse signed zeros among positives
        a = np.where(rng.random(n) < 0.01, np.where(rng.random(n) < 0.5, -0.0, 0.0),
                     1 + rng.random(n)).astype(np.float32)
    else:
        a = rng.random(n).astype(np.float32)
        a[rng.integers(0, n, max(1, n // 50))] = a.min()
    v, rf_log, lanes = CFGS[int(rng.integers(0, len(CFGS)))]
    tmin = (2 if v.startswith("cl") else 1) << rf_log
    t = int(rng.choice([0, tmin, tmin + 1, 32, 64, 100, 1024, 1 << 14, 1 << 16, n + 5]))
    t = max(t, tmin) if t else 0
    q = int(rng.integers(1, 8000))
    law = int(rng.integers(0, 3))
    if law == 0:
        length = rng.integers(1, n + 1, q)
    elif law == 1:
        length = np.minimum(n, np.exp(rng.normal(np.log(max(2.0, n ** 0.5)), 1.5, q)).astype(np.int64) + 1)
    else:
        length = np.minimum(n, rng.integers(1, 80, q))
    lo = (rng.random(q) * (n - length + 1)).astype(np.int64)
    qs = np.stack([lo, lo + length - 1], 1).astype(np.uint32)
    return a, qs, v, rf_log, lanes, t


@pytest.mark.parametrize("seed", range(6))
def test_random_cases(cuda, seed):
    import torch
    rng = np.random.default_rng(1000 + seed)
    for c in range(40):
        a, qs, v, rf_log, lanes, t = _case(rng)
        dv = torch.from_numpy(a).to(cuda)
        dq = torch.from_numpy(qs.view(np.int32)).to(cuda)
        with R.Hierarchy(dv, variant=v, t=t, rf_log=rf_log, lanes=lanes) as h:
            m = h.query(dq).cpu().numpy()
            i, m2 = h.query_idx(dq, with_min=True)
            i = i.cpu().numpy().view(np.uint32)
            m2 = m2.cpu().numpy()
        em = oracle.rmq_min(a, qs, 8).astype(np.float32)
        ei = oracle.rmq_argmin(a, qs, 8)
        what = f"seed {seed} case {c}: n={a.size} {v} rf={1 << rf_log} lanes={lanes} t={t}"
        assert m.tobytes() == em.tobytes(), what
        assert m2.tobytes() == em.tobytes(), what
        assert np.array_equal(i, ei), what
