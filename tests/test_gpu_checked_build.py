"""The GPU suites again, against the bounds-checked build of the library
(librmq_gb300_checked.so: RMQ_DEBUG_BOUNDS=1, every level load of the query
kernels checked before it is made, out-of-level loads counted and skipped):
every result must still be exact and the count must be zero.  This stands in
for compute-sanitizer, which is not available where the library is tested.

Runs the suites in a child pytest process pointed at the checked library
(RMQ_GB300_LIB); the child's session end reads the count (tests/conftest.py).
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]
CHECKED = ROOT / "gpu-rmq_gb300" / "librmq_gb300_checked.so"
SUITES = ["tests/test_gpu_parity.py", "tests/test_gpu_fuzz.py", "tests/test_gpu_wide.py", "tests/test_gpu_batch.py",
          "tests/test_gpu_host_buffers.py", "tests/test_gpu_serve.py", "tests/test_zz_no_alloc.py"]


def test_suites_under_bounds_checked_build(cuda):
    assert CHECKED.exists(), "the bounds-checked library was not built"
    env = dict(os.environ, RMQ_GB300_LIB=str(CHECKED), RMQ_EXPECT_CHECKED_LIB="1")
    # The full-size workloads are left out (they repeat the same code paths at
    # sizes that would only lengthen the run).
    cmd = [sys.executable, "-m", "pytest", *SUITES, "-m", "gpu", "-x", "-q", "-p", "no:cacheprovider",
           "-k", "not full_size and not beyond_2_pow_32"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=1800)
    tail = r.stdout[-4000:] + r.stderr[-2000:]
    assert r.returncode == 0, tail
    assert "out-of-level loads 0" in r.stdout, tail
    ran = re.search(r"(\d+) passed", r.stdout)
    assert ran is not None and int(ran.group(1)) >= 150, tail  # the suites really ran
    print(ran.group(0), "under the bounds-checked build, no out-of-level load")
