"""The server's arena bookkeeping (gpu-rmq_gb300/csrc/rmq_arena.h, host only)
on the CPU: a seeded random sequence of allocations and releases against a
byte-exact model.  Checks first fit (lowest offset that holds the request),
256-byte granules, no overlap of live ranges, and that released ranges merge
so the free list always covers exactly the bytes not in use; and the
eviction choice (least recently used among resident, built, unpinned
arrays other than the one being admitted)."""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
G = 256


def _round(x: int) -> int:
    return (x + G - 1) // G * G


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("arena") / "arena_harness"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", str(ROOT / "gpu-rmq_gb300" / "csrc"),
                    str(ROOT / "tests" / "arena_harness.cpp"), "-o", str(exe)], check=True)
    return exe


def _run(exe, lines):
    out = subprocess.run([str(exe)], input="\n".join(lines) + "\n", capture_output=True, text=True, check=True)
    return out.stdout.splitlines()


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_arena_against_model(harness, seed):
    rng = np.random.default_rng(seed)
    size = 1 << 20
    cmds = [f"i {size}"]
    # Model: the live ranges, chosen by first fit over the free bytes.
    live = {}
    expect = []
    plan = []
    for step in range(600):
        if live and rng.random() < 0.45:
            off = int(rng.choice(sorted(live)))
            plan.append(("r", off, live.pop(off)))
        else:
            want = int(rng.integers(1, 40000))
            b = _round(want)
            # first fit: lowest offset whose free gap holds b
            used = sorted((o, o + l) for o, l in live.items())
            cur, got = 0, None
            for o, e in used + [(size, size)]:
                if o - cur >= b:
                    got = cur
                    break
                cur = max(cur, e)
            plan.append(("a", want, got))
            if got is not None:
                live[got] = b
        plan.append(("f",))
    # replay on the harness, checking each answer
    out_lines = _run(harness, cmds + [
        (f"a {p[1]}" if p[0] == "a" else f"r {p[1]} {p[2]}" if p[0] == "r" else "f") for p in plan])
    it = iter(out_lines)
    live2 = {}
    for p in plan:
        if p[0] == "a":
            line = next(it)
            if p[2] is None:
                assert line == "full"
            else:
                assert line == f"ok {p[2]}", (line, p)
                live2[p[2]] = _round(p[1])
        elif p[0] == "r":
            live2.pop(p[1])
        else:
            parts = next(it).split()
            assert parts[0] == "free"
            ranges = [(int(parts[2 + 2 * i]), int(parts[3 + 2 * i])) for i in range(int(parts[1]))]
            # free ranges: sorted, disjoint, not adjacent (merged), and exactly the complement
            covered = sorted(ranges + [(o, l) for o, l in live2.items()])
            pos = 0
            for o, l in covered:
                assert o == pos and l > 0, (o, pos)
                pos = o + l
            assert pos == size
            for (o1, l1), (o2, _) in zip(ranges, ranges[1:]):
                assert o1 + l1 < o2  # neighbours were merged


def test_lru_victim_against_model(harness):
    rng = np.random.default_rng(5)
    cmds, expect = [], []
    for _ in range(300):
        n = int(rng.integers(0, 12))
        rows = [(int(rng.random() < 0.7), int(rng.random() < 0.8), int(rng.random() < 0.2),
                 int(rng.integers(0, 50))) for _ in range(n)]
        except_ = int(rng.integers(0, max(1, n)))
        cmds.append(f"v {except_} {n} " + " ".join(f"{a} {b} {c} {d}" for a, b, c, d in rows))
        best, oldest = None, None
        for i, (res, rdy, pins, last) in enumerate(rows):
            if i != except_ and res and rdy and pins == 0 and (oldest is None or last < oldest):
                best, oldest = i, last
        expect.append("victim none" if best is None else f"victim {best}")
    assert _run(harness, cmds) == expect
