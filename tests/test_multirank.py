"""Host logic of the N > 1 bench path on CPU with world_size-2 gloo ranks.

Every rank answers its own replica (no collective on the data path); the only
cross-rank steps are the barrier and the max-over-ranks reduction of the
elapsed time, from which value = all ranks' queries / max time.
"""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank: int, ws: int, port: int, q: int, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    sys.path.insert(0, str(root))
    import numpy as np
    import bench
    from oracle import oracle

    bench.dist_init(ws, "gloo")
    wsz, rk, local = bench.dist_env()
    # each rank answers its own replica: different seeds -> different inputs
    a, qs = bench.make_inputs(4096, q, -1, 42 + rk)
    res = oracle.rmq_min(a, qs, 1)
    bench.barrier(ws)
    elapsed = 1.0 + rk  # rank 1 is the slow one
    t_max = bench.max_over_ranks(elapsed, ws)
    value = bench.aggregate_value(q, 3, t_max * 1e3, ws)
    out.put((rk, wsz, float(res.sum()), t_max, value))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks_weak_scaling():
    ws, q = 2, 1000
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, ws, port, q, out)) for r in range(ws)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(out.get(timeout=10) for _ in range(ws))
    assert [g[0] for g in got] == [0, 1] and all(g[1] == ws for g in got)
    assert got[0][2] != got[1][2]  # replicas differ (per-rank seeds)
    assert all(g[3] == 2.0 for g in got)  # max over ranks seen by both
    assert got[0][4] == pytest.approx(ws * q * 3 / 2.0)  # all ranks' queries / max time


def test_reference_arm_rank_nonzero_does_nothing(capsys):
    import bench
    args = bench.parse_args(["--impl", "reference", "--n", "4096", "--q", "1024", "--steps", "1"])
    bench.run_reference(args, 2, 1)
    assert capsys.readouterr().out == ""
