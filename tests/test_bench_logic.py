"""Host logic of bench.py on the CPU: the algorithmic-bytes model against a
brute-force sector count, the served trace generator, the workload names and
the traffic figures read from the committed ncu summaries."""
from __future__ import annotations

import numpy as np
import pytest

import bench


def _sectors_brute(l: int, r: int, n: int) -> int:
    """Distinct 32-byte sectors of the level-0 array that the canonical
    descent (rf_c = 32) reads for the inclusive query [l, r]."""
    e = r + 1
    rf = 32
    if e - l <= 2 * rf or n <= 64:
        pos = range(l, e)
    else:
        nl = (l + rf - 1) // rf * rf
        pr = e // rf * rf
        pos = list(range(l, nl)) + list(range(pr, e))
    return len({p // 8 for p in pos})


def test_level0_sectors_matches_brute_force():
    rng = np.random.default_rng(0)
    for n in (1, 7, 64, 65, 1000, 1 << 20):
        q = 500
        length = rng.integers(1, n + 1, q)
        l = (rng.random(q) * (n - length + 1)).astype(np.int64)
        qs = np.stack([l, l + length - 1], 1).astype(np.uint32)
        got = bench.level0_sectors(qs, n)
        want = [_sectors_brute(int(a), int(b), n) for a, b in qs]
        assert np.array_equal(got, want), n


def _coarse_brute(l: int, r: int, n: int) -> int:
    """Sectors of levels >= 1 read by the canonical descent (rf 32, t 64),
    walking the levels one query at a time."""
    rf, t = 32, 64
    sizes = [n]
    while len(sizes) < 20 and sizes[-1] > t:
        sizes.append(-(-sizes[-1] // rf))
    top = len(sizes) - 1
    lo, e, k, total = l, r + 1, 0, 0
    while k < top and e - lo > 2 * rf:
        nl = -(-lo // rf) * rf
        pr = e // rf * rf
        if k > 0:
            total += len({p // 8 for p in range(lo, nl)}) + len({p // 8 for p in range(pr, e)})
        lo, e, k = nl // rf, pr // rf, k + 1
    if k > 0:
        total += len({p // 8 for p in range(lo, e)})
    return total


def test_coarse_sectors_matches_brute_force():
    rng = np.random.default_rng(2)
    for n in (1, 64, 65, 5000, 1 << 16, 1 << 22):
        q = 400
        length = np.minimum(rng.integers(1, n + 1, q), n)
        length[: q // 4] = np.minimum(np.exp(rng.uniform(0, np.log(n + 1), q // 4)).astype(np.int64) + 1, n)
        l = (rng.random(q) * (n - length + 1)).astype(np.int64)
        qs = np.stack([l, l + length - 1], 1).astype(np.uint32)
        got = bench.coarse_sectors(qs, n)
        want = [_coarse_brute(int(a), int(b), n) for a, b in qs]
        assert np.array_equal(got, want), n


def test_algorithmic_bytes_counts_query_and_results():
    qs = np.array([[0, 0], [0, 63], [5, 200]], dtype=np.uint32)
    s = int(bench.level0_sectors(qs, 1000).sum())
    assert bench.algorithmic_bytes(qs, 1000, True, True) == 3 * (8 + 4 + 4) + 32 * s
    assert bench.algorithmic_bytes(qs, 1000, True, False) == 3 * (8 + 4) + 32 * s


def test_serve_trace_shape():
    rng = np.random.default_rng(1)
    sizes = [1 << 16, 1 << 18, 1 << 20]
    ev, lr, n_of = bench.serve_trace(rng, sizes, 0.05, 20000.0, 0.05, 3)
    t = ev["t_arrival_s"]
    assert (np.diff(t) >= 0).all() and t[-1] < 0.05
    reg = ev["kind"] == 1
    assert 0 < reg.sum() < 0.2 * ev.size
    assert len(n_of) == len(sizes) + int(reg.sum())
    req = ~reg
    q = ev["q"][req]
    assert (q >= 1).all() and (q <= 1 << 16).all()
    assert lr.shape[0] == int(q.sum())
    for i in np.flatnonzero(req)[:50]:
        o, c, aid = int(ev["q_offset"][i]), int(ev["q"][i]), int(ev["array_id"][i])
        part = lr[o:o + c]
        assert (part[:, 0] <= part[:, 1]).all() and (part[:, 1] < n_of[aid]).all()
        # an array registered by the trace is named only after its registration
        if aid >= len(sizes):
            k = aid - len(sizes)
            assert np.flatnonzero(reg)[k] < i


def test_workload_names_follow_the_length_law():
    a = bench.parse_args(["--lr", "-8", "--ties", "0.01", "--n", str(1 << 28)])
    w = bench.workload_config(a)["workload"]
    assert "n=2^28" in w and "1 % of entries" in w and "one third each" in w
    a = bench.parse_args([])
    w = bench.workload_config(a)["workload"]
    assert "n=2^26" in w and "q=2^26" in w and "ln 2^13" in w


@pytest.mark.parametrize("tag", ["vl-rf8", "cl-rf8-g2", "cl-rf16-g4"])
def test_traffic_figures_are_committed(tag):
    v = bench.traffic_per_query(tag)
    assert v is not None and 100.0 < v < 400.0


def test_reference_arm_line_on_cpu():
    """`bench.py --impl reference` runs the oracle's CPU scan on the host
    only, and prints one JSON line with the contract's keys."""
    import json
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    out = subprocess.run([sys.executable, str(root / "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "3", "--n", "65536", "--q", "4096", "--lr", "-1",
                          "--ref-step-queries", "1024"],
                         capture_output=True, text=True, timeout=300, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["steps"] == 2
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["workload"].startswith("plain single array")


def test_reference_arm_maps_no_product_library():
    """The reference arm gets its inputs from the oracle's own generators:
    no library of the product package is mapped into its process."""
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    code = ("import sys; sys.path.insert(0, %r); import bench; "
            "bench.main(['--impl', 'reference', '--steps', '1', '--warmup', '3', '--n', '4096', '--q', '512', "
            "'--lr', '-7', '--ref-step-queries', '128']); "
            "maps = open('/proc/self/maps').read(); "
            "print('PRODUCT-MAPPED' if 'gpu-rmq_gb300' in maps else 'NO-PRODUCT-LIBRARY')" % str(root))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip().splitlines()[-1] == "NO-PRODUCT-LIBRARY"


def test_sub_record_selection():
    assert bench.selected_sub_records("none") == []
    assert bench.selected_sub_records("all") == bench.SUB_RECORDS
    assert bench.selected_sub_records("c1_n2e20,served_c5") == ["c1_n2e20", "served_c5"]
    with pytest.raises(SystemExit):
        bench.selected_sub_records("c9")


def test_cpu_list_and_numa_maps_parsing():
    assert bench._cpulist("0-3,8,10-11") == {0, 1, 2, 3, 8, 10, 11}
    a = np.ones(1 << 20, dtype=np.float32)  # a mapping of its own
    nodes = bench.buffer_nodes(a.ctypes.data)
    assert isinstance(nodes, dict)
