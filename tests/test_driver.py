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


def run(*args, cwd=None):
    return subprocess.run([str(RTXRMQ), *map(str, args)], capture_output=True, text=True, cwd=cwd,
                          timeout=120)


def test_help_and_bad_arguments():
    r = run()
    assert r.returncode != 0 and "run as ./rtxrmq" in r.stderr
    assert run(100, 10, 200, 0).returncode != 0  # lr > n
    assert run(100, 10, -9, 0, "--seed", 1).returncode != 0  # unknown law
    r = run(100, 10, -1, 16)
    assert r.returncode != 0 and "variant cl" in r.stderr  # reference-only kernel ids
    assert run(100, 10, -1, 5).returncode != 0  # not in this driver


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
    row = lines[1].split(",")
    assert len(row) == len(lines[0].split(","))
    assert row[-5] == "-1"  # checkResult: no check ran


@pytest.mark.gpu
@pytest.mark.parametrize("alg,extra", [
    (22, ["--variant", "vl"]), (22, ["--variant", "cl"]), (122, ["--variant", "auto"]),
    (122, ["--variant", "cl", "--rf_log", "5", "--lanes", "16"]), (2, []), (102, []),
])
@pytest.mark.parametrize("check", ["--check", "--randTrivialCheck", "--trivialCheck"])
def test_gpu_algorithms_pass_checks(cuda, tmp_path, alg, extra, check):
    csv = tmp_path / "t.csv"
    r = run(1 << 20, 1 << 16, -6, alg, "--seed", 913, "--reps", 3, "--log_bs", 10, check,
            f"--save-time={csv}", *extra)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    assert "pass" in r.stdout and "failed" not in r.stdout
    row = csv.read_text().splitlines()[1].split(",")
    code = int(row[-5])
    assert code == {"--check": 1, "--trivialCheck": 3, "--randTrivialCheck": 5}[check]


@pytest.mark.gpu
def test_gpu_large_mixed_ties_check(cuda):
    r = run(1 << 24, 1 << 20, -8, 122, "--seed", 7, "--reps", 2, "--log_bs", 6, "--ties", "0.01",
            "--randTrivialCheck")
    assert r.returncode == 0 and "pass" in r.stdout, r.stdout[-2000:]
