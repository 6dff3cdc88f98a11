"""The rtxrmq driver on CPU: argument handling, CPU algorithms against the
oracle through --save-input-data output, CSV schema."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import PKG
from oracle import oracle

import rmq_gb300 as R

RTXRMQ = PKG / "driver" / "rtxrmq"


def _row(csv, i=0):
    """Row i of a CSV written by rtxrmq, as {column: text}."""
    lines = csv.read_text().splitlines()
    head = lines[0].split(",")
    row = lines[1 + i].split(",")
    assert len(row) == len(head), (head, row)
    return dict(zip(head, row))


def run(*args, cwd=None):
    return subprocess.run([str(RTXRMQ), *map(str, args)], capture_output=True, text=True, cwd=cwd,
                          timeout=120)


def test_help_and_bad_arguments():
    r = run()
    assert r.returncode != 0 and "./rtxrmq <n> <q> <lr> <alg>" in r.stderr
    assert run(100, 10, 200, 0).returncode != 0  # lr > n
    assert run(100, 10, -9, 0, "--seed", 1).returncode != 0  # unknown law
    r = run(100, 10, -1, 16)
    assert r.returncode != 0 and "variant cl" in r.stderr  # reference-only kernel ids
    assert run(100, 10, -1, 5).returncode != 0  # not in this driver
    r = run(100, 10, -1, 22, "--variant", "cl-fast")
    assert r.returncode != 0 and "unknown --variant" in r.stderr


@pytest.mark.parametrize("alg", [0, 100])
def test_cpu_algorithms_and_csv(tmp_path, alg):
    n, q, lr, seed = 5000, 777, -6, 913
    csv = tmp_path / "out.csv"
    r = run(n, q, lr, alg, "--seed", seed, "--nt", 2, "--reps", 2, "--save-input-data",
            "--data-dir", tmp_path, f"--save-time={csv}")
    assert r.returncode == 0, r.stderr
    # cached inputs are the reference generator's, byte for byte
    a = np.fromfile(tmp_path / f"array_n-{n}_seed-{seed}.bin", dtype=np.float32)
    assert a.tobytes() == R.gen_array(n, seed).tobytes()
    qs = np.fromfile(next(tmp_path.glob("queries_*.bin")), dtype=np.uint32).reshape(-1, 2)
    assert np.array_equal(qs, R.gen_queries(q, lr, n, seed))
    lines = csv.read_text().splitlines()
    assert lines[0].startswith("dev,alg,nt,reps,n,bs,nb,q,lr,GPU_BSIZE,CG_GROUP_SIZE,CG_MEM_ALIGNMENT,timestamp,t,q/s")
    row = _row(csv)
    assert row["checkResult"] == "-1"  # no check ran
    assert row["mode"] == "cpu" and row["bs"] == "1" and row["nb"] == "0"


@pytest.mark.gpu
@pytest.mark.parametrize("alg,extra", [
    (22, ["--variant", "vl"]), (22, ["--variant", "cl"]), (122, ["--variant", "auto"]),
    (122, ["--variant", "cl", "--rf_log", "5", "--lanes", "16"]), (2, []), (102, []),
    (22, ["--variant", "cl-noshuffle", "--rf_log", "5", "--lanes", "16"]), (122, ["--variant", "cl-tile"]),
    (122, ["--variant", "cl-atomic", "--lanes", "8"]), (122, ["--variant", "vl-short"]),
])
@pytest.mark.parametrize("check", ["--check", "--randTrivialCheck", "--trivialCheck"])
def test_gpu_algorithms_pass_checks(cuda, tmp_path, alg, extra, check):
    csv = tmp_path / "t.csv"
    r = run(1 << 20, 1 << 16, -6, alg, "--seed", 913, "--reps", 3, "--log_bs", 10, check,
            f"--save-time={csv}", *extra)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "pass" in r.stdout and "failed" not in r.stdout
    row = _row(csv)
    code = int(row["checkResult"])
    assert code == {"--check": 1, "--trivialCheck": 3, "--randTrivialCheck": 5}[check]


@pytest.mark.gpu
def test_gpu_large_mixed_ties_check(cuda):
    r = run(1 << 24, 1 << 20, -8, 122, "--seed", 7, "--reps", 2, "--log_bs", 6, "--ties", "0.01",
            "--randTrivialCheck")
    assert r.returncode == 0 and "pass" in r.stdout, r.stdout[-2000:]


def test_reference_sweep_command_line_cpu(tmp_path):
    """A command line of the reference's sweep (scripts/perf-benchmark-exp.sh:48-49:
    --nb, --reps, --nt, --dev, --save-time=, --seed) plus its other flags
    (--log_build_threshold, --save-power) is accepted; the row keeps the
    reference's column meanings."""
    csv = tmp_path / "sweep.csv"
    r = run(1 << 12, 1 << 10, -1, 0, "--nb", 1 << 6, "--reps", 1, "--nt", 2, "--dev", 0,
            f"--save-time={csv}", "--seed", 27722, "--log_build_threshold=3", "--save-power")
    assert r.returncode == 0, r.stderr
    row = _row(csv)
    assert row["alg"] == "[CPU] BASE" and row["n"] == str(1 << 12) and row["q"] == str(1 << 10)
    assert row["lr"] == "-1" and row["nt"] == "2" and row["reps"] == "1"
    assert row["bs"] == "1" and row["nb"] == "0"  # the reference resets both for this algorithm
    assert float(row["q/s"]) > 0 and row["checkResult"] == "-1"


@pytest.mark.gpu
@pytest.mark.parametrize("variant,rf_log,lanes,size_log,amount_log", [
    ("vl", 3, 0, 0, 1), ("cl", 3, 2, 1, 2), ("cl", 5, 16, 4, 1)])
def test_gpu_hierarchy_row_columns(cuda, tmp_path, variant, rf_log, lanes, size_log, amount_log):
    """Hierarchy rows: scan_threshold from --nb as the reference computes it,
    XXX_CG_SIZE_LOG = log2(lanes) (0 for VL), XXX_CG_AMOUNT_LOG = log2(rf /
    lanes) (VL: log2(rf / 4)), the level buffer in outbuffer, the argmin
    positions in tempbuffer, and the roofline columns."""
    csv = tmp_path / "h.csv"
    n = 1 << 20
    extra = ["--lanes", lanes] if lanes else []
    r = run(n, 1 << 16, -7, 122, "--nb", 1 << 12, "--reps", 2, "--variant", variant, "--rf_log", rf_log,
            f"--save-time={csv}", "--seed", 5, "--randTrivialCheck", *extra)
    assert r.returncode == 0 and "pass" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
    row = _row(csv)
    assert row["scan_threshold"] == str(n >> 12)  # 2^ceil(log2(n / nb))
    assert int(row["XXX_CG_SIZE_LOG"]) == size_log and int(row["XXX_CG_AMOUNT_LOG"]) == amount_log
    info = R.plan_layout(n, n >> 12, rf_log, variant)
    lvl_mb = info.level_offset[info.num_levels - 1] + info.level_size[info.num_levels - 1]
    assert float(row["outbuffer"]) > 0 and abs(float(row["outbuffer"]) - float(row["tempbuffer"])) < 1e-6
    assert float(row["outbuffer"]) >= 4 * lvl_mb / 1e6 - 1e-6
    assert float(row["hbm_GBps"]) > 0 and 0 < float(row["roofline_frac"]) < 2
    assert row["mode"] == "plain" and int(row["checkResult"]) == 5
