#!/usr/bin/env python3
"""Benchmark of the GB300 hierarchical RMQ path.

Headline workload (N = 1): the plain single-array configuration — n = 2^26
fp32 values uniform in [0, 1), q = 2^26 inclusive queries with lengths
clamp(round(exp(N(ln 2^13, 1))), 1, n) and l uniform in [0, n - len]; every
query returns its fp32 minimum and its int32 argmin (ties to the lowest
index).  One step is one pass of the query kernel over all q queries with the
array, the hierarchy and the queries resident in HBM.  The inputs (1 GiB of
queries and values, 512 MiB of outputs) exceed the 129 MB L2, so no flush is
needed between steps (smaller workloads are timed step by step with L2
flushed in between).  The line also carries the roofline of the query
kernel (HBM, and L2 against an L2 read rate measured here), the end-to-end
figure through rmq_query_idx_host on page-locked host buffers, the
reference's own GPU kernels timed on the same inputs, the CPU baseline and
the SM clocks sampled during the timed region.

The default run adds `sub_records`, each with its own value, ms_per_step,
roofline, parity sample and clocks:
  mixture_n2e26  n = q = 2^26, 1 % of entries tied at the minimum, lengths one
                 third each uniform [1, n], lognormal(2^13, 1), lognormal(2^5,
                 0.7), t = 64 (the mixed-length target: >= 0.60 of HBM peak)
  c3_n2e28       n = 2^28 with 1 % ties, q = 2^27, the same mixture, t = 64
  c1_n2e20       n = 2^20, q = 2^16, lengths uniform [1, n] (the reference's
                 CPU case), L2 flushed between steps, against the L2 read rate
  batched_c4     4096 arrays (batched form vs a per-array loop of the plain
                 kernels with buffers allocated up front)
  served_c5      the serving loop on a Poisson trace (p50 / p99 latency;
                 capacity vs a per-request loop of the plain kernel)

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--mode plain|batched|serve] [--sub-records all|none|a,b]
                  [--n N --q Q --lr L --t T --ties F]

Under torchrun each rank builds and queries its own replica on its own GPU
(no collective on the data path); value = all ranks' queries / max-over-ranks
time ("weak" scaling).  The reference arm (--impl reference) times the
reference's CPU brute-force scan (restated in oracle/, inputs from the
oracle's own generators) on the host cores.
"""
from __future__ import annotations

import argparse
import gc
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "gpu-rmq_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "RMQ queries/s"
UNIT = "queries/s"
CANON_RF_LOG = 5   # canonical descent for algorithmic bytes: rf_c = 32 (128-B lines)
SECTOR = 32


# ---------------------------------------------------------------------------
# Algorithmic bytes (implementation independent): per query, 8 B of query,
# 4 B of min, 4 B of argmin, plus the 32-B sectors of the input array that
# the canonical descent (rf = 32) reads at level 0: the sectors of [l, r] when
# len <= 64, else those of [l, ceil32(l)) and [floor32(r+1), r+1).
# ---------------------------------------------------------------------------
def level0_sectors(qs: np.ndarray, n: int) -> np.ndarray:
    l = qs[:, 0].astype(np.int64)
    r = qs[:, 1].astype(np.int64)
    e = r + 1
    rf = 1 << CANON_RF_LOG
    short = (e - l) <= 2 * rf
    if n <= 64:
        short[:] = True
    s_short = (r >> 3) - (l >> 3) + 1
    nl = (l + rf - 1) & ~(rf - 1)
    pr = e & ~(rf - 1)
    left = np.where(nl > l, ((nl - 1) >> 3) - (l >> 3) + 1, 0)
    right = np.where(e > pr, (r >> 3) - (pr >> 3) + 1, 0)
    return np.where(short, s_short, left + right)


CANON_T = 64  # scan threshold of the canonical hierarchy for the L2 byte model


def coarse_sectors(qs: np.ndarray, n: int) -> np.ndarray:
    """Per query, the 32-B sectors of levels >= 1 that the canonical descent
    (rf_c = 32, t_c = 64) reads: its boundary pieces while it descends, then
    the final piece where it stops.  Those levels live in L2, so these bytes
    go against L2, not HBM."""
    rf = 1 << CANON_RF_LOG
    sizes = [n]
    while len(sizes) < 20 and sizes[-1] > CANON_T:
        sizes.append((sizes[-1] + rf - 1) // rf)
    top = len(sizes) - 1
    l = qs[:, 0].astype(np.int64)
    e = qs[:, 1].astype(np.int64) + 1
    out = np.zeros(l.shape[0], dtype=np.int64)
    live = np.ones(l.shape[0], dtype=bool)  # still descending at level k
    for k in range(top + 1):
        if k > 0:
            # final piece [l, e) at level k for queries that stop here
            stop = live & ~((k < top) & (e - l > 2 * rf))
            fin = stop & (e > l)
            out += np.where(fin, ((e - 1) >> 3) - (l >> 3) + 1, 0)
            live &= ~stop
        go = live & (k < top) & (e - l > 2 * rf)
        if k == 0:
            live &= go
        nl = (l + rf - 1) & ~(rf - 1)
        pr = e & ~(rf - 1)
        if k > 0:
            left = np.where(go & (nl > l), ((nl - 1) >> 3) - (l >> 3) + 1, 0)
            right = np.where(go & (e > pr), ((e - 1) >> 3) - (pr >> 3) + 1, 0)
            out += left + right
        l = np.where(go, nl >> CANON_RF_LOG, l)
        e = np.where(go, pr >> CANON_RF_LOG, e)
    return out


def algorithmic_bytes(qs: np.ndarray, n: int, with_min: bool, with_idx: bool) -> int:
    per_q = 8 + (4 if with_min else 0) + (4 if with_idx else 0)
    return int(per_q * qs.shape[0] + SECTOR * int(level0_sectors(qs, n).sum()))


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def traffic_per_query(kernel_tag: str) -> float | None:
    """DRAM bytes per query of the query kernel from the committed ncu summary
    (a line `traffic_bytes_per_query[<tag>]: X`), or None."""
    for p in sorted((ROOT / "profiles").glob("*.md")):
        for line in p.read_text().splitlines():
            key = f"traffic_bytes_per_query[{kernel_tag}]:"
            if line.strip().startswith(key):
                try:
                    return float(line.split(":", 1)[1].strip().split()[0])
                except ValueError:
                    return None
    return None


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.25)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# distributed helpers (one process per GPU; timing reduction only)
# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws: int, backend: str):
    if ws <= 1:
        return None
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend=backend)
    return dist


def max_over_ranks(x: float, ws: int, device=None) -> float:
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_value(q: int, steps: int, max_ms: float, ws: int) -> float:
    """Whole-job throughput: every rank's queries over the slowest rank's time."""
    return ws * q * steps / (max_ms / 1e3)


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------------------
# ---------------------------------------------------------------------------
# inputs
# ---------------------------------------------------------------------------
def make_inputs(n: int, q: int, lr: int, seed: int, ties: float = 0.0):
    """The GPU arm's inputs, from the library's host generators."""
    import rmq_gb300 as R
    a = R.gen_array(n, seed)
    if ties > 0.0:
        R.plant_min_ties(a, ties, seed)
    qs = R.gen_queries(q, lr, n, seed)
    return a, qs


def make_inputs_oracle(n: int, q: int, lr: int, seed: int, ties: float = 0.0):
    """The reference arm's inputs, from the oracle's own restatement of the
    same generators (bit-identical to make_inputs; no product library is
    loaded)."""
    from oracle import oracle
    a = oracle.gen_array(n, seed)
    if ties > 0.0:
        oracle.plant_min_ties(a, ties, seed)
    return a, oracle.gen_queries(q, lr, n, seed)


def algorithmic_bytes_chunked(qs: np.ndarray, n: int, chunk: int = 1 << 22) -> int:
    """algorithmic_bytes (min + argmin) over a large query set, in chunks."""
    return sum(algorithmic_bytes(qs[i:i + chunk], n, True, True) for i in range(0, qs.shape[0], chunk))


def cpu_baseline(a: np.ndarray, qs: np.ndarray, budget_s: float, with_idx: bool = True) -> dict:
    """The reference's brute-force scan as it runs it (oracle restatement of
    cpu_rmq / cpu_rmq_idx, src/cpu_methods.h:18-77, one OpenMP parallel for
    with the default schedule) on all host threads, over consecutive chunks
    of the same query set until `budget_s` of wall time is used."""
    from oracle import oracle
    threads = oracle.max_threads()
    chunk = 1 << 14
    done = 0
    t0 = time.perf_counter()
    while done < qs.shape[0] and time.perf_counter() - t0 < budget_s:
        part = np.ascontiguousarray(qs[done: done + chunk])
        oracle.cpu_rmq(a, part, threads)
        if with_idx:
            oracle.cpu_rmq_idx(a, part, threads)
        done += part.shape[0]
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {done} of the {qs.shape[0]} queries (min{' + argmin' if with_idx else ''}), "
                      f"{dt:.1f} s wall on {threads} threads",
            "schedule": "cpu_rmq / cpu_rmq_idx restated with the reference's default OpenMP schedule "
                        "(src/cpu_methods.h:28, :65)"}


def run_reference(args, ws, rank):
    """Reference arm: the reference's CPU scan (alg 0 + alg 100, as
    cpu_rmq / cpu_rmq_idx run it) on the host cores, rank 0 only; each step is
    a bounded sample.  Inputs come from the oracle's generators, so no
    product library is loaded."""
    if rank != 0:
        return
    from oracle import oracle
    a, qs = make_inputs_oracle(args.n, args.q, args.lr, args.seed, args.ties)
    threads = oracle.max_threads()
    per_step = args.ref_step_queries
    rng = np.random.default_rng(args.seed)
    times = []
    for i in range(args.warmup + args.steps):
        start = int(rng.integers(0, max(1, qs.shape[0] - per_step)))
        part = np.ascontiguousarray(qs[start: start + per_step])
        t0 = time.perf_counter()
        oracle.cpu_rmq(a, part, threads)
        oracle.cpu_rmq_idx(a, part, threads)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    ms = 1e3 * statistics.mean(times)
    value = per_step / (ms / 1e3)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(args, "not applicable (host CPU run, a bounded sample of the queries per step)"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{per_step} consecutive queries per step (random offset), "
                                   f"min + argmin brute-force scan on {threads} threads",
                         "schedule": "cpu_rmq / cpu_rmq_idx restated with the reference's default "
                                     "OpenMP schedule (src/cpu_methods.h:28, :65)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


LENGTH_LAWS = {
    -1: "len uniform in [1,n]",
    -2: "len lognormal(median n^0.6, sigma 0.3)",
    -3: "len lognormal(median n^0.3, sigma 0.3)",
    -4: "len lognormal(median n/2^8, sigma 0.3)",
    -5: "len lognormal(median n/2^15, sigma 0.3)",
    -6: "len mixture of the laws -1/-2/-3",
    -7: "len=clamp(round(exp(N(ln 2^13,1))),1,n)",
    -8: "len one third each uniform [1,n], lognormal(2^13, 1.0), lognormal(2^5, 0.7), clamped",
}


# Inputs + outputs below this (2x the 129 MB L2) are timed with L2 flushed
# between steps.
L2_FLUSH_BELOW = 258 << 20


def workload_name(n: int, q: int, lr: int, ties: float) -> str:
    law = LENGTH_LAWS.get(lr, f"len = {lr}" if lr > 0 else f"length law {lr}")
    tie = f" with {100 * ties:g} % of entries set to the global minimum" if ties > 0 else ""
    return (f"plain single array: n=2^{np.log2(n):g} fp32 uniform[0,1){tie}, q=2^{np.log2(q):g} queries, "
            f"{law}, l uniform in [0,n-len]; min + argmin per query")


def workload_config(args, l2_note: str = "inputs larger than L2 (no flush)") -> dict:
    return {"workload": workload_name(args.n, args.q, args.lr, args.ties),
            "n": args.n, "q": args.q, "lr_code": args.lr, "seed": args.seed, "ties": args.ties,
            "variant": args.variant, "scan_threshold": args.t, "rf_log": args.rf_log, "lanes": args.lanes,
            "l2": l2_note, "parallelism": f"replicas x{dist_env()[0]}"}


# ---------------------------------------------------------------------------
# L2 read rate (measured here; no datasheet figure exists for GB300)
# ---------------------------------------------------------------------------
_L2_PEAK = None


def l2_peak(dev) -> dict:
    """Rate at which the SMs read L2-resident 32-byte sectors with the query
    kernels' load form (rmq_measure_l2_read over a 32 MiB buffer: in address
    order, and at hashed sector positions), best of 3 runs of 50 passes."""
    global _L2_PEAK
    if _L2_PEAK is None:
        import torch
        import rmq_gb300 as R
        buf = torch.ones(1 << 23, dtype=torch.float32, device=dev)  # 32 MiB
        seq = max(R.measure_l2_read(buf, 50, False) for _ in range(3))
        rnd = max(R.measure_l2_read(buf, 50, True) for _ in range(3))
        del buf
        _L2_PEAK = {"GBps": seq, "random_sectors_GBps": rnd,
                    "how": "rmq_measure_l2_read: 32 MiB buffer, 256-bit loads with L1 bypassed, 64 warps/SM, "
                           "best of 3 x 50 passes (sequential sectors = peak; hashed sectors for context)"}
    return _L2_PEAK


# ---------------------------------------------------------------------------
# plain single-array measurement (headline and sub-records)
# ---------------------------------------------------------------------------
def parity_sample(a: np.ndarray, qs: np.ndarray, out_min, out_idx, seed: int, size: int = 1 << 14) -> bool:
    """The timed outputs on a seeded sample of queries against the oracle's
    sparse table (checked against the brute-force scan in the CPU tests)."""
    import rmq_gb300 as R
    from oracle import oracle
    samp = R.sample_indices(qs.shape[0], size, seed).astype(np.int64)
    import torch
    idx_t = torch.from_numpy(samp).to(out_min.device)
    got_m = out_min[idx_t].cpu().numpy()
    got_i = out_idx[idx_t].cpu().numpy().view(np.uint32)
    exp_m, exp_i = oracle.Sparse(a).query(np.ascontiguousarray(qs[samp]))
    return bool(got_m.tobytes() == exp_m.tobytes() and np.array_equal(got_i, exp_i))


def plain_measure(n, q, lr, ties, t, seed, args, dev, stream, ws, *, tag_suffix="", l2_bound=False,
                  keep=False):
    """Builds the hierarchy over a generated array and times `args.steps`
    launches of the min + argmin query kernel over q generated queries (CUDA
    events on the launching stream; L2 flushed between steps when the inputs
    fit in it).  Returns the record and, with keep, the buffers for the
    headline's extra measurements."""
    import torch
    import rmq_gb300 as R

    a, qs = make_inputs(n, q, lr, seed, ties)
    dv = torch.from_numpy(a).to(dev)
    dq = torch.from_numpy(qs.view(np.int32)).to(dev)
    out_min = torch.empty(q, dtype=torch.float32, device=dev)
    out_idx = torch.empty(q, dtype=torch.int32, device=dev)
    sh = stream.cuda_stream
    # The first build also loads the kernels (lazy module loading); the
    # reported build time is that of a second, warm build.
    R.Hierarchy(dv, variant=args.variant, t=t, rf_log=args.rf_log, lanes=args.lanes,
                l2_persist=args.l2_persist, stream=stream).close()
    h = R.Hierarchy(dv, variant=args.variant, t=t, rf_log=args.rf_log, lanes=args.lanes,
                    l2_persist=args.l2_persist, stream=stream)
    info = h.info()
    torch.cuda.synchronize()
    lr_ptr, idx_ptr, min_ptr = int(dq.data_ptr()), int(out_idx.data_ptr()), int(out_min.data_ptr())

    def step():
        st = h.query_idx_raw(lr_ptr, q, idx_ptr, min_ptr, sh)
        if st != 0:
            raise R.RMQError(st, "rmq_query_idx")

    footprint = 4 * n + int(info.level_bytes) + 16 * q
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev) if footprint < L2_FLUSH_BELOW else None
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clocks:
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                if flush is not None:
                    flush.fill_(k & 0xFF)
                ev[2 * k].record(stream)
                step()
                ev[2 * k + 1].record(stream)
        torch.cuda.synchronize()
    barrier(ws)
    per_launch = [ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(args.steps)]
    total_ms = sum(per_launch) if flush is not None else ev[0].elapsed_time(ev[2 * args.steps - 1])
    total_ms = max_over_ranks(total_ms, ws, dev)
    value = aggregate_value(q, args.steps, total_ms, ws)
    l2_note = ("L2 flushed between steps (512 MiB write, untimed)" if flush is not None
               else "inputs larger than L2 (no flush)")

    # minimum-only pass (same kernel family, no argmin)
    with torch.cuda.stream(stream):
        for _ in range(max(1, args.warmup)):
            h.query_raw(lr_ptr, q, min_ptr, sh)
        em = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
        for k in range(args.steps):
            if flush is not None:
                flush.fill_(k & 0xFF)
            em[2 * k].record(stream)
            h.query_raw(lr_ptr, q, min_ptr, sh)
            em[2 * k + 1].record(stream)
    torch.cuda.synchronize()
    min_ms = (sum(em[2 * k].elapsed_time(em[2 * k + 1]) for k in range(args.steps)) if flush is not None
              else em[0].elapsed_time(em[2 * args.steps - 1]))
    min_only_qps = q * args.steps / (min_ms / 1e3)
    # restore the argmin + min outputs (the minimum-only pass rewrote out_min)
    with torch.cuda.stream(stream):
        step()
    torch.cuda.synchronize()
    parity = parity_sample(a, qs, out_min, out_idx, seed)

    peaks = measured_peaks()
    kernel_ms = statistics.mean(per_launch)
    alg_bytes = algorithmic_bytes_chunked(qs, n)
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    vname = {1: "cl", 2: "vl", 3: "cl-noshuffle", 4: "cl-tile", 5: "cl-atomic",
             6: "vl-short"}.get(int(info.variant), "cl")
    is_vl = info.variant in (2, 6)
    tag = f"{vname}-rf{1 << info.rf_log}" if is_vl else f"{vname}-rf{1 << info.rf_log}-g{info.lanes}"
    tpq = traffic_per_query(tag + tag_suffix)
    l2p = l2_peak(dev)
    l2_sample = qs[: 1 << 20]
    l2_per_q = SECTOR * float(coarse_sectors(l2_sample, n).mean()) if l2_sample.shape[0] else 0.0
    l2_achieved = l2_per_q * q / (kernel_ms / 1e3) / 1e9
    l2 = {"algorithmic_bytes_per_query": l2_per_q, "achieved_GBps": l2_achieved, "peak": l2p["GBps"],
          "frac": l2_achieved / l2p["GBps"], "peak_random_sectors_GBps": l2p["random_sectors_GBps"],
          "peak_source": "measured here (" + l2p["how"] + ")",
          "sample": f"first {l2_sample.shape[0]} queries",
          "model": "32 B x sectors of levels >= 1 read by the canonical descent (rf 32, t 64)"}
    kernel = f"query_{'vl' if is_vl else 'cl'}_kernel (argmin+min), {tag}"
    if 3 <= info.variant <= 5:
        kernel += " (the reference's ablation of CL as a work distribution)"
    if info.variant == 6:
        kernel += " (short-query form: level-0 winners taken in phase 1)"
    if l2_bound:
        # every input of this workload fits in L2: the same algorithmic bytes
        # go against the L2 read rate (inputs are flushed from L2 between steps)
        roofline = {"bound": "l2", "achieved": achieved, "peak": l2p["GBps"], "unit": "GB/s",
                    "frac": achieved / l2p["GBps"], "traffic": (tpq * q) if tpq is not None else None,
                    "peak_source": "measured here (" + l2p["how"] + ")",
                    "algorithmic_bytes_per_launch": alg_bytes, "kernel": kernel, "kernel_ms_mean": kernel_ms,
                    "hbm_frac": achieved / peaks["hbm_gbs"]}
    else:
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                    "frac": achieved / peaks["hbm_gbs"], "traffic": (tpq * q) if tpq is not None else None,
                    "peak_source": f"{peaks['source']} (MEASURED_PEAKS.json hbm_gbs, copy burst)",
                    "algorithmic_bytes_per_launch": alg_bytes, "kernel": kernel, "kernel_ms_mean": kernel_ms,
                    "l2": l2}
    build_bytes = 4 * n + 8 * sum(info.sizes()[1:])
    rec = {"value": value, "unit": UNIT, "ms_per_step": total_ms / args.steps, "steps": args.steps,
           "warmup": args.warmup, "workload": workload_name(n, q, lr, ties),
           "n": n, "q": q, "lr_code": lr, "ties": ties, "seed": seed, "scan_threshold": t, "l2": l2_note,
           "roofline": roofline, "clocks": clocks.summary(), "parity_sample_ok": parity,
           "parity_sample": "2^14 seeded queries of the timed outputs vs the oracle's sparse table",
           "min_only_queries_per_s": min_only_qps, "gpu_launches": args.steps,
           "hierarchy": {"variant": vname, "rf": 1 << info.rf_log,
                         "t": int(info.scan_threshold), "levels": int(info.num_levels),
                         "lanes": int(info.lanes), "level_bytes": int(info.level_bytes),
                         "build_ms": float(info.build_ms),
                         "build_GBps": build_bytes / (float(info.build_ms) / 1e3) / 1e9
                         if info.build_ms > 0 else None}}
    ctx = None
    if keep:
        ctx = {"a": a, "qs": qs, "dv": dv, "dq": dq, "h": h, "out_min": out_min, "out_idx": out_idx,
               "min_only_qps": min_only_qps, "clocks": clocks, "per_launch": per_launch,
               "total_ms": total_ms, "l2_note": l2_note}
    else:
        h.close()
        del dv, dq, out_min, out_idx, flush
        gc.collect()
        torch.cuda.empty_cache()
    return rec, ctx


PLAIN_SUBS = {
    "mixture_n2e26": {"n": 1 << 26, "q": 1 << 26, "lr": -8, "ties": 0.01, "t": 64, "tag": "-mixture",
                      "target": {"what": "plain kernel at n = 2^26 with mixed query lengths: "
                                         "roofline.frac >= 0.60 of the HBM peak", "frac_at_least": 0.60}},
    "c3_n2e28": {"n": 1 << 28, "q": 1 << 27, "lr": -8, "ties": 0.01, "t": 64, "tag": "-n2e28"},
    "c1_n2e20": {"n": 1 << 20, "q": 1 << 16, "lr": -1, "ties": 0.0, "t": 64, "tag": "-n2e20", "l2": True},
}
SUB_RECORDS = list(PLAIN_SUBS) + ["batched_c4", "served_c5"]


def selected_sub_records(spec: str) -> list[str]:
    if spec in ("", "none"):
        return []
    if spec == "all":
        return list(SUB_RECORDS)
    names = [x.strip() for x in spec.split(",") if x.strip()]
    bad = [x for x in names if x not in SUB_RECORDS]
    if bad:
        raise SystemExit(f"bench.py: unknown sub-records {bad}; choose from {SUB_RECORDS}")
    return names


def run_ours(args, ws, rank, local):
    import torch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist_init(ws, "nccl")
    stream = torch.cuda.Stream(device=dev)

    rec, ctx = plain_measure(args.n, args.q, args.lr, args.ties, args.t, args.seed + rank, args, dev, stream, ws,
                             keep=True)
    a, qs, h = ctx["a"], ctx["qs"], ctx["h"]
    q = qs.shape[0]

    # --- end to end: pinned host queries -> device -> host results -------------
    e2e = run_e2e(args, h, qs, dev, ws, ctx["out_idx"], ctx["out_min"], ctx["dq"])
    ref_style = reference_style_timing(h, ctx, args, stream)
    sweep = t_sweep(ctx, args, dev, stream) if args.t_sweep else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(a, qs, args.cpu_budget)

    # The reference's own CL / VL kernels (compiled from its sources for
    # sm_103a, oracle/_ref) on the same GPU and inputs: minima only, as the
    # reference has no hierarchical argmin.
    reference_gpu = None
    if not args.no_reference_gpu:
        from oracle import ref_gpu
        if not ref_gpu.available():
            reference_gpu = {"unavailable": "reference kernels not built (reference sources absent at build)"}
        elif args.n % 4:
            reference_gpu = {"unavailable": "n % 4 != 0 (the reference VL kernel reads whole float4s)"}
        else:
            reference_gpu = {}
            ours_min = ctx["out_min"].clone()
            for variant, t in (("cl", 64), ("vl", 32), ("cl", args.t), ("vl", args.t)):
                key = f"{variant}_t{t}"
                if key in reference_gpu:
                    continue
                with torch.cuda.stream(stream):
                    qps, ref_out = ref_gpu.time_reference(ctx["dv"], ctx["dq"], variant, t, steps=args.steps,
                                                          warmup=3)
                reference_gpu[key] = {"queries_per_s": qps,
                                      "minima_equal_ours": bool(torch.equal(ref_out.view(torch.int32),
                                                                            ours_min.view(torch.int32)))}
                del ref_out
            best = max(v["queries_per_s"] for v in reference_gpu.values())
            reference_gpu["best_queries_per_s"] = best
            reference_gpu["ours_min_only_vs_best"] = ctx["min_only_qps"] / best
            reference_gpu["ours_min_argmin_vs_best"] = rec["value"] / ws / best

    line = {
        "metric": METRIC, "value": rec["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": rec["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generators; no public dataset)",
        "config": workload_config(args, ctx["l2_note"]),
        "roofline": rec["roofline"],
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": rec["clocks"],
        "gpu_launches": args.steps,
        "parity_sample_ok": rec["parity_sample_ok"],
        "min_only_queries_per_s": rec["min_only_queries_per_s"],
        "reference_gpu": reference_gpu,
        "hierarchy": rec["hierarchy"],
        "reference_style_timing": ref_style,
    }
    if sweep is not None:
        line["t_sweep"] = sweep
    h.close()
    del ctx
    gc.collect()
    torch.cuda.empty_cache()

    subs = {}
    for name in selected_sub_records(args.sub_records):
        t0 = time.perf_counter()
        try:
            if name in PLAIN_SUBS:
                c = PLAIN_SUBS[name]
                r, _ = plain_measure(c["n"], c["q"], c["lr"], c["ties"], c["t"], args.seed + rank, args, dev,
                                     stream, ws, tag_suffix=c["tag"], l2_bound=c.get("l2", False))
                if "target" in c:
                    r["target"] = dict(c["target"], met=bool(r["roofline"]["frac"] >= c["target"]["frac_at_least"]))
            elif name == "batched_c4":
                r = batched_record(args, ws, rank, dev)
            else:
                r = served_record(args, ws, rank, dev)
        except Exception as exc:  # a failed sub-record is reported, the headline stands
            r = {"error": f"{type(exc).__name__}: {exc}"}
        r["wall_s"] = time.perf_counter() - t0
        subs[name] = r
        gc.collect()
        torch.cuda.empty_cache()
    if subs:
        line["sub_records"] = subs
        line["targets"] = targets_summary(subs)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def reference_style_timing(h, ctx, args, stream) -> dict:
    """The reference's own way of timing a query run (src/xxx.h:276-283): the
    host clock around each launch followed by a device synchronisation, one
    launch per repetition.  Reported beside the CUDA-event figure."""
    import torch
    q = ctx["qs"].shape[0]
    lr_ptr, idx_ptr, min_ptr = int(ctx["dq"].data_ptr()), int(ctx["out_idx"].data_ptr()), int(ctx["out_min"].data_ptr())
    sh = stream.cuda_stream
    times = []
    for k in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = h.query_idx_raw(lr_ptr, q, idx_ptr, min_ptr, sh)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        if st != 0:
            raise RuntimeError(f"rmq_query_idx failed: {st}")
        if k >= args.warmup:
            times.append(dt * 1e3)
    med = statistics.median(times)
    return {"ms_median": med, "ms_mean": statistics.mean(times), "queries_per_s_median": q / (med / 1e3),
            "reps": len(times),
            "what": "host clock around one launch + device synchronisation per repetition, the reference's "
                    "timed loop (src/xxx.h:276-283); `value` uses CUDA events"}


T_SWEEP = (32, 64, 1 << 10, 1 << 12, 1 << 14, 1 << 16)


def t_sweep(ctx, args, dev, stream) -> dict:
    """The headline workload's queries over hierarchies built with other scan
    thresholds (the reference's `t`; the paper uses 64 for CL, 32 for VL):
    queries/s by CUDA events per launch and whether the results equal the
    headline's bit for bit."""
    import torch
    import rmq_gb300 as R
    q = ctx["qs"].shape[0]
    dq = ctx["dq"]
    ref_min, ref_idx = ctx["out_min"], ctx["out_idx"]
    out_min = torch.empty_like(ref_min)
    out_idx = torch.empty_like(ref_idx)
    sh = stream.cuda_stream
    steps = max(1, min(args.steps, 5))
    out = {}
    for t in T_SWEEP:
        try:
            h = R.Hierarchy(ctx["dv"], variant=args.variant, t=t, rf_log=args.rf_log, lanes=args.lanes,
                            stream=stream)
        except R.RMQError as exc:  # below the variant's minimum t (CL: 2 rf, VL: rf)
            out[str(t)] = {"unsupported": R.strerror(exc.status)}
            continue
        info = h.info()
        args_ptrs = (int(dq.data_ptr()), q, int(out_idx.data_ptr()), int(out_min.data_ptr()), sh)
        with torch.cuda.stream(stream):
            for _ in range(2):
                if h.query_idx_raw(*args_ptrs) != 0:
                    raise RuntimeError("rmq_query_idx failed")
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        with torch.cuda.stream(stream):
            ev[0].record(stream)
            for _ in range(steps):
                h.query_idx_raw(*args_ptrs)
            ev[1].record(stream)
        torch.cuda.synchronize()
        ms = ev[0].elapsed_time(ev[1]) / steps
        same = bool(torch.equal(out_idx, ref_idx) and torch.equal(out_min.view(torch.int32), ref_min.view(torch.int32)))
        out[str(t)] = {"queries_per_s": q / (ms / 1e3), "ms": ms, "levels": int(info.num_levels),
                       "results_equal_headline": same}
        h.close()
    del out_min, out_idx
    return {"by_t": out, "steps": steps, "variant": args.variant,
            "what": "the headline's queries and array, hierarchy rebuilt per scan threshold t"}


def targets_summary(subs: dict) -> dict:
    """The benchmark spec's targets next to the measured figures."""
    out = {}
    m = subs.get("mixture_n2e26", {})
    if "roofline" in m:
        out["plain_mixture_n2e26_frac"] = {"value": m["roofline"]["frac"], "target": 0.60,
                                          "met": m["roofline"]["frac"] >= 0.60}
    b = subs.get("batched_c4", {})
    if "speedup_vs_plain_loop" in b:
        out["batched_vs_per_array_plain_loop"] = {"value": b["speedup_vs_plain_loop"], "target": 3.0,
                                                  "met": b["speedup_vs_plain_loop"] >= 3.0,
                                                  "loop": b["loop_plain_kernels"]["what"]}
    s = subs.get("served_c5", {})
    if "speedup_capacity_vs_loop" in s:
        out["served_capacity_vs_per_request_loop"] = {"value": s["speedup_capacity_vs_loop"], "target": 3.0,
                                                      "met": s["speedup_capacity_vs_loop"] >= 3.0,
                                                      "loop": s["loop_plain_kernel"]["what"]}
    return out


# ---------------------------------------------------------------------------
# host memory placement for the end-to-end figure
# ---------------------------------------------------------------------------
def _read(path: str) -> str | None:
    try:
        return Path(path).read_text().strip()
    except OSError:
        return None


def _cpulist(text: str) -> set[int]:
    cpus = set()
    for part in text.split(","):
        part = part.strip()
        if not part:
            continue
        if "-" in part:
            a, b = part.split("-")
            cpus.update(range(int(a), int(b) + 1))
        else:
            cpus.add(int(part))
    return cpus


def gpu_host_node(gpu_index: int) -> dict:
    """The host NUMA node the GPU's PCI function reports (sysfs), and that
    node's CPUs."""
    out = {"gpu_pci_bus_id": None, "gpu_numa_node": None, "node_cpus": None}
    try:
        bus = subprocess.run(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=pci.bus_id",
                              "--format=csv,noheader"], capture_output=True, text=True, timeout=20).stdout.strip()
    except (OSError, subprocess.TimeoutExpired):
        return out
    if not bus:
        return out
    # nvidia-smi prints an 8-digit domain ("00000009:01:00.0"); sysfs uses 4
    dom, rest = bus.split(":", 1)
    sysfs = f"{int(dom, 16):04x}:{rest}".lower()
    out["gpu_pci_bus_id"] = sysfs
    node = _read(f"/sys/bus/pci/devices/{sysfs}/numa_node")
    if node is not None and node.lstrip("-").isdigit():
        out["gpu_numa_node"] = int(node)
        if int(node) >= 0:
            cpus = _read(f"/sys/devices/system/node/node{int(node)}/cpulist")
            if cpus:
                out["node_cpus"] = sorted(_cpulist(cpus))
    return out


def buffer_nodes(addr: int) -> dict:
    """Pages per NUMA node of the mapping holding host address `addr`
    (/proc/self/numa_maps)."""
    maps = _read("/proc/self/maps") or ""
    start = None
    for line in maps.splitlines():
        lo, hi = (int(x, 16) for x in line.split()[0].split("-"))
        if lo <= addr < hi:
            start = lo
            break
    if start is None:
        return {}
    for line in (_read("/proc/self/numa_maps") or "").splitlines():
        fields = line.split()
        if fields and int(fields[0], 16) == start:
            return {f.split("=")[0]: int(f.split("=")[1]) for f in fields if f[:1] == "N" and "=" in f}
    return {}


def run_e2e(args, h, qs, dev, ws, out_idx, out_min, d_q) -> dict:
    """Same metric through the C ABI with host buffers: every step is one
    rmq_query_idx_host call on page-locked host buffers (queries in, min +
    argmin out); with page-locked buffers the library's kernel reads the
    queries from and writes the results to host memory directly.  The results
    must equal those of the device-buffer call."""
    import torch
    q = qs.shape[0]
    # Page-locked buffers on the GPU's host node: the thread is bound to that
    # node's CPUs while it allocates (first touch places the pages there) and
    # while it runs the end-to-end steps; the placement is recorded.
    place = gpu_host_node(dev.index)
    prev_aff = os.sched_getaffinity(0) if hasattr(os, "sched_getaffinity") else None
    bound = False
    if prev_aff is not None and place["node_cpus"]:
        local = set(place["node_cpus"]) & prev_aff
        if local:
            os.sched_setaffinity(0, local)
            bound = True
    h_q = torch.from_numpy(qs.view(np.int32).reshape(-1)).pin_memory()
    h_min = torch.empty(q, dtype=torch.float32).pin_memory()
    h_idx = torch.empty(q, dtype=torch.int32).pin_memory()
    h_min.fill_(0.0)
    h_idx.fill_(0)
    place["thread_bound_to_node_cpus"] = bound
    place["buffer_pages_by_node"] = {"queries": buffer_nodes(int(h_q.data_ptr())),
                                     "argmin": buffer_nodes(int(h_idx.data_ptr())),
                                     "min": buffer_nodes(int(h_min.data_ptr()))}

    def one_pass():
        st = h.query_idx_host_raw(int(h_q.data_ptr()), q, int(h_idx.data_ptr()), int(h_min.data_ptr()))
        if st != 0:
            raise RuntimeError(f"rmq_query_idx_host failed: {st}")

    for _ in range(max(1, args.warmup)):
        one_pass()
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one_pass()
    torch.cuda.synchronize()
    dt = max_over_ranks(time.perf_counter() - t0, ws, dev)
    same = bool(torch.equal(h_idx, out_idx.cpu()) and torch.equal(h_min.view(torch.int32), out_min.cpu().view(torch.int32)))
    link = host_link_rates(h_q, h_idx, h_min, out_idx, out_min)
    step_s = dt / args.steps
    link["achieved_GBps"] = 16 * q / step_s / 1e9
    link["frac_of_duplex"] = link["achieved_GBps"] / link["duplex_GBps"]
    link["kernel_ms_by_buffer_placement"] = placement_breakdown(h, q, d_q, out_idx, out_min, h_q, h_idx, h_min)
    link["numa"] = place
    if bound:
        os.sched_setaffinity(0, prev_aff)
    return {"value": ws * q * args.steps / dt, "unit": UNIT, "h2d_bytes_per_step": 8 * q,
            "d2h_bytes_per_step": 8 * q,
            "api": "rmq_query_idx_host on page-locked host buffers (kernel reads / writes host memory)",
            "kernel_launches_per_step": 1, "results_equal_device_call": same, "host_link": link}


def placement_breakdown(h, q, d_q, d_idx, d_min, h_q, h_idx, h_min, reps: int = 5) -> dict:
    """The query kernel's time (CUDA events, ms per launch) with queries and
    results each in device memory or in page-locked host memory (the kernel
    reaching host memory over the link), through rmq_query_idx: where the
    end-to-end step's time over the device-resident one goes.  Run after the
    timed region; the result buffers receive the same results again."""
    import torch
    out = {}
    for name, lq, oi, om in (("device queries, device results", d_q, d_idx, d_min),
                             ("host queries, device results", h_q, d_idx, d_min),
                             ("device queries, host results", d_q, h_idx, h_min),
                             ("host queries, host results", h_q, h_idx, h_min)):
        def launch():
            st = h.query_idx_raw(int(lq.data_ptr()), q, int(oi.data_ptr()), int(om.data_ptr()))
            if st != 0:
                raise RuntimeError(f"rmq_query_idx failed: {st}")
        launch()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            launch()
        e1.record()
        torch.cuda.synchronize()
        out[name] = e0.elapsed_time(e1) / reps
    return out


def host_link_rates(h_q, h_idx, h_min, d_idx, d_min, reps: int = 3) -> dict:
    """The host link's own rates for the end-to-end step's bytes, by copy
    engine: the queries host -> device, the two result arrays device ->
    host, and both directions at once on two streams (the end-to-end step's
    floor is its 16 bytes per query at the duplex rate).  Run after the
    timed region; the result buffers receive the device results again."""
    import torch
    d_q = torch.empty_like(h_q, device=d_idx.device)
    s_up, s_down = torch.cuda.Stream(), torch.cuda.Stream()
    cur = torch.cuda.current_stream()

    def up():
        d_q.copy_(h_q, non_blocking=True)

    def down():
        h_idx.copy_(d_idx, non_blocking=True)
        h_min.copy_(d_min, non_blocking=True)

    def both():
        s_up.wait_stream(cur)
        s_down.wait_stream(cur)
        with torch.cuda.stream(s_up):
            up()
        with torch.cuda.stream(s_down):
            down()
        cur.wait_stream(s_up)
        cur.wait_stream(s_down)

    def rate(fn, nbytes):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return nbytes / (e0.elapsed_time(e1) / reps / 1e3) / 1e9

    # The same copies split into four chunks on four streams each way (more
    # copy engines at work): whether one engine per direction limits the rate.
    k = 4
    ups, downs = [torch.cuda.Stream() for _ in range(k)], [torch.cuda.Stream() for _ in range(k)]
    cq, cr = h_q.numel() // k, h_idx.numel() // k

    def split(direction_up: bool, direction_down: bool):
        def fn():
            for i in range(k):
                lo_q, hi_q = i * cq, (h_q.numel() if i == k - 1 else (i + 1) * cq)
                lo_r, hi_r = i * cr, (h_idx.numel() if i == k - 1 else (i + 1) * cr)
                if direction_up:
                    ups[i].wait_stream(cur)
                    with torch.cuda.stream(ups[i]):
                        d_q[lo_q:hi_q].copy_(h_q[lo_q:hi_q], non_blocking=True)
                if direction_down:
                    downs[i].wait_stream(cur)
                    with torch.cuda.stream(downs[i]):
                        h_idx[lo_r:hi_r].copy_(d_idx[lo_r:hi_r], non_blocking=True)
                        h_min[lo_r:hi_r].copy_(d_min[lo_r:hi_r], non_blocking=True)
            for i in range(k):
                cur.wait_stream(ups[i])
                cur.wait_stream(downs[i])
        return fn

    nq = h_q.numel() * 4
    nr = h_idx.numel() * 4 + h_min.numel() * 4
    out = {"h2d_GBps": rate(up, nq), "d2h_GBps": rate(down, nr), "duplex_GBps": rate(both, nq + nr),
           "h2d_GBps_4_streams": rate(split(True, False), nq),
           "d2h_GBps_4_streams": rate(split(False, True), nr),
           "duplex_GBps_4_streams": rate(split(True, True), nq + nr),
           "what": "copy-engine rates of the same buffers (page-locked host <-> device), "
                   "one stream per direction and four chunks on four streams per direction"}
    del d_q
    return out


# ---------------------------------------------------------------------------
# batched form (4096 arrays)
# ---------------------------------------------------------------------------
def batched_record(args, ws, rank, dev) -> dict:
    """Batched workload: 4096 arrays, sizes log-uniform in [2^10, 2^22],
    uniform [0, 1) values, min(4 x size, 2^20) queries per array with lengths
    lognormal(median sqrt(size), sigma 1) clamped to [1, size].  One step =
    build of every array + every query (one CUDA graph launch), inputs
    resident.  Compared with the per-array loop of the plain kernels over the
    same preallocated buffers (rmq_batch_run_per_array: per array the
    single-array build and query launches, one stream, no synchronisation),
    and with a per-array loop through the public API (rmq_build, which
    allocates and waits, + rmq_query_idx)."""
    import torch
    import rmq_gb300 as R
    from oracle import oracle

    rng = np.random.default_rng(args.seed + rank)
    A = args.batch_arrays
    sizes = np.exp(rng.uniform(np.log(2.0 ** 10), np.log(2.0 ** 22), A)).astype(np.uint64)
    offs, total = R.pack_offsets(sizes)
    qcounts = np.minimum(4 * sizes, np.uint64(1 << 20))
    qo = np.zeros(A + 1, dtype=np.uint64)
    qo[1:] = np.cumsum(qcounts)
    Q = int(qo[-1])
    values = torch.empty(total, dtype=torch.float32, device=dev)
    R.gen_values_device(values, args.seed + 1000 * rank)
    lr = torch.empty((Q, 2), dtype=torch.int32, device=dev)
    for a in range(A):
        s0, s1 = int(qo[a]), int(qo[a + 1])
        R.gen_queries_device(lr[s0:s1], int(sizes[a]), 1, float(np.sqrt(float(sizes[a]))), 1.0,
                             args.seed * 7919 + a)
    out_min = torch.empty(Q, dtype=torch.float32, device=dev)
    out_idx = torch.empty(Q, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.synchronize()

    b = R.Batch(values, offs, sizes, t=64, stream=stream)
    b.set_queries(lr, qo, out_idx, out_min, stream=stream)
    tuned = b.autotune(stream=stream)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            b.run(stream=stream)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
    barrier(ws)
    with ClockSampler(dev.index) as clocks:
        ev[0].record(stream)
        for _ in range(args.steps):
            b.run(stream=stream)
        ev[1].record(stream)
        torch.cuda.synchronize()
    total_ms = max_over_ranks(ev[0].elapsed_time(ev[1]), ws, dev)
    value = aggregate_value(Q, args.steps, total_ms, ws)
    # build-only and query-only timings (same kernels, outside the graph)
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record(stream)
    b.build(stream=stream)
    e1.record(stream)
    b.query(stream=stream)
    e2.record(stream)
    torch.cuda.synchronize()
    build_ms, query_ms = e0.elapsed_time(e1), e1.elapsed_time(e2)

    # parity: a seeded sample of arrays against the CPU oracle
    parity = True
    for a in rng.choice(A, size=min(A, 8), replace=False):
        o, n = int(offs[a]), int(sizes[a])
        s0, s1 = int(qo[a]), int(qo[a + 1])
        x = values[o:o + n].cpu().numpy()
        qh = lr[s0:s1].cpu().numpy().view(np.uint32)
        parity &= out_min[s0:s1].cpu().numpy().tobytes() == oracle.rmq_min(x, qh).tobytes()
        parity &= np.array_equal(out_idx[s0:s1].cpu().numpy().view(np.uint32), oracle.rmq_argmin(x, qh))

    # comparator: the per-array loop of the plain kernels (C side, buffers
    # allocated up front, one stream, no synchronisation between arrays)
    ref_min, ref_idx = out_min.clone(), out_idx.clone()
    out_min.fill_(-1.0)
    out_idx.fill_(-1)
    loop_steps = max(1, min(args.steps, 5))
    with torch.cuda.stream(stream):
        b.run_per_array(stream=stream)
    torch.cuda.synchronize()
    loop_same = bool(torch.equal(out_idx, ref_idx) and torch.equal(out_min.view(torch.int32),
                                                                   ref_min.view(torch.int32)))
    e0.record(stream)
    for _ in range(loop_steps):
        b.run_per_array(stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    loop_ms = e0.elapsed_time(e1) / loop_steps
    loop_value = Q / (loop_ms / 1e3)
    del ref_min, ref_idx

    # a per-array loop through the public API (allocating rmq_build + query)
    hs = []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for a in range(A):
        o, n = int(offs[a]), int(sizes[a])
        h = R.Hierarchy(values[o:o + n], variant="vl", t=64, stream=stream)
        s0, s1 = int(qo[a]), int(qo[a + 1])
        h.query_idx_raw(int(lr[s0:s1].data_ptr()), s1 - s0, int(out_idx[s0:s1].data_ptr()),
                        int(out_min[s0:s1].data_ptr()), stream)
        hs.append(h)
    torch.cuda.synchronize()
    loop_api_s = time.perf_counter() - t0
    for h in hs:
        h.close()
    b.close()
    del values, lr, out_min, out_idx

    return {
        "metric": "RMQ queries/s (batched: build + queries of every array per step)", "value": value,
        "unit": UNIT, "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "workload": f"batched: {A} arrays, sizes log-uniform [2^10, 2^22], "
                    "queries min(4 size, 2^20) lognormal(sqrt(size), 1.0); min + argmin",
        "arrays": A, "total_values": total, "total_queries": Q, "seed": args.seed,
        "l2": "inputs larger than L2 (no flush)", "data": "synthetic (device counter-based generators)",
        "autotuned": {"scan_threshold": int(tuned.scan_threshold), "query_block": int(tuned.query_block),
                      "class_threshold": [int(x) for x in tuned.class_threshold],
                      "class_upper_entries": ["2^14", "2^18", "any"],
                      "query_ms": float(tuned.query_ms)},
        "build_ms": build_ms, "query_ms": query_ms,
        "loop_plain_kernels": {"value": loop_value, "ms_per_step": loop_ms, "steps": loop_steps,
                               "results_equal_batched": loop_same,
                               "what": "rmq_batch_run_per_array: per array the plain single-array build and "
                                       "query launches over the batch's preallocated buffers, one stream, "
                                       "no synchronisation (C side)"},
        "loop_public_api": {"value": Q / loop_api_s, "seconds": loop_api_s,
                            "what": "per array from Python: rmq_build (allocates, builds, waits) + rmq_query_idx"},
        "speedup_vs_plain_loop": value / loop_value,
        "speedup_vs_loop_public_api": value / (Q / loop_api_s),
        "clocks": clocks.summary(), "gpu_launches": 3 * args.steps, "parity_sample_ok": bool(parity),
    }


def run_batched(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    dist_init(ws, "nccl")
    rec = batched_record(args, ws, rank, torch.device("cuda", local))
    line = {"metric": rec.pop("metric"), "value": rec.pop("value"), "unit": rec.pop("unit"), "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": rec.pop("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": rec.pop("data"), "config": {"workload": rec.pop("workload"), "arrays": rec["arrays"],
                                                "total_values": rec["total_values"],
                                                "total_queries": rec["total_queries"], "seed": args.seed,
                                                "l2": rec.pop("l2")}}
    line.update(rec)
    if rank == 0:
        print(json.dumps(line), flush=True)


def serve_trace(rng, sizes, seconds, rate, reg_frac, seed, max_log2: float = 26.0):
    """Poisson request stream: arrivals at `rate`/s for `seconds`; a fraction
    reg_frac registers a new array (size law of the resident ones), the rest
    are requests naming a registered array, with 1..2^16 queries (log-uniform)
    of lognormal(2^13, 1) lengths clamped to the array."""
    import rmq_gb300 as R
    gaps = rng.exponential(1.0 / rate, int(seconds * rate * 1.5) + 16)
    t = np.cumsum(gaps)
    t = t[t < seconds]
    E = t.size
    ev = np.zeros(E, dtype=R.TRACE_DTYPE)
    ev["t_arrival_s"] = t
    n_of = list(sizes)
    is_reg = rng.random(E) < reg_frac
    qcount = np.exp(rng.uniform(0.0, np.log(2.0 ** 16), E)).astype(np.int64).clip(1, 1 << 16)
    off = 0
    req_n = np.zeros(E, dtype=np.int64)
    for i in range(E):
        if is_reg[i]:
            n = int(np.exp(rng.uniform(np.log(2.0 ** 16), np.log(2.0 ** max_log2))))
            ev["kind"][i] = 1
            ev["n"][i] = n
            ev["seed"][i] = seed * 1000003 + len(n_of)
            n_of.append(n)
        else:
            aid = int(rng.integers(0, len(n_of)))
            ev["array_id"][i] = aid
            ev["q_offset"][i] = off
            ev["q"][i] = qcount[i]
            req_n[i] = n_of[aid]
            off += int(qcount[i])
    lr = np.empty((off, 2), dtype=np.uint32)
    for i in np.flatnonzero(~is_reg):
        q, n, o = int(ev["q"][i]), int(req_n[i]), int(ev["q_offset"][i])
        length = np.rint(np.exp(rng.normal(np.log(8192.0), 1.0, q))).clip(1, n).astype(np.int64)
        l = (rng.random(q) * (n - length + 1)).astype(np.int64)
        lr[o:o + q, 0] = l
        lr[o:o + q, 1] = l + length - 1
    return ev, lr, n_of


# ---------------------------------------------------------------------------
# served form
# ---------------------------------------------------------------------------
def served_record(args, ws, rank, dev) -> dict:
    """Serving workload: 256 resident arrays (sizes log-uniform [2^16, 2^26],
    device-generated values), a Poisson stream of 20k requests/s for
    --serve-seconds, 5 % of them registering a new array, 64 GiB HBM budget
    with LRU eviction; p50/p99 request latency and queries/s.  Capacity: the
    same requests on the initial arrays issued at once, against the C-side
    per-request loop of the plain kernel (rmq_serve_serial_loop: per request
    rmq_query_idx_host on a prebuilt handle, waited for before the next)."""
    import torch
    import rmq_gb300 as R
    from oracle import oracle

    phase = {}
    tp = time.perf_counter()

    def mark(name):
        nonlocal tp
        now = time.perf_counter()
        phase[name] = round(now - tp, 3)
        tp = now

    rng = np.random.default_rng(args.seed + rank)
    top = float(args.serve_max_log2)
    sizes = [int(np.exp(rng.uniform(np.log(2.0 ** 16), np.log(2.0 ** top)))) for _ in range(args.serve_arrays)]
    seed_of = lambda a: args.seed * 1000003 + a  # noqa: E731  (the trace uses the same rule)
    ev, lr_pageable, n_of = serve_trace(rng, sizes, args.serve_seconds, 20000.0, 0.05, args.seed, top)
    req = ev["kind"] == 0
    Q = int(ev["q"][req].sum())
    mark("trace")
    # The request buffers are page-locked (the server then reads the queries
    # and writes the results in place), and written once up front: the replay
    # measures the server, not first-touch page faults of fresh host memory.
    lr_t = torch.from_numpy(lr_pageable.view(np.int32).reshape(-1)).pin_memory()
    lr = lr_t.numpy().view(np.uint32).reshape(-1, 2)
    out_i_t = torch.ones(Q, dtype=torch.int32).pin_memory()
    out_m_t = torch.ones(Q, dtype=torch.float32).pin_memory()
    out_i = out_i_t.numpy().view(np.uint32)
    out_m = out_m_t.numpy()
    mark("pin_buffers")

    # Warm-up on a throwaway server (a 0.2 s trace over 32 small arrays): the
    # first serving run of a process otherwise carries a cold tail (first
    # kernel launches, first batches of the dispatcher).
    wrng = np.random.default_rng(args.seed + 7919)
    wsizes = [int(np.exp(wrng.uniform(np.log(2.0 ** 12), np.log(2.0 ** 20)))) for _ in range(32)]
    wev, wlr, _ = serve_trace(wrng, wsizes, 0.2, 20000.0, 0.05, args.seed + 7919)
    with R.Server(hbm_budget_bytes=1 << 30, slots=args.serve_slots, t=64,
                  query_threads=args.serve_threads) as wsrv:
        for a, n in enumerate(wsizes):
            wsrv.register_generated(n, args.seed + 7919 + a)
        wq = int(wev["q"][wev["kind"] == 0].sum())
        wsrv.replay(wev, wlr, np.empty(wq, np.uint32), np.empty(wq, np.float32))
    mark("warmup_server")

    srv = R.Server(hbm_budget_bytes=int(args.serve_budget_gib * (1 << 30)), slots=args.serve_slots, t=64,
                   query_threads=args.serve_threads)
    for a, n in enumerate(sizes):
        srv.register_generated(n, seed_of(a))
    warm = np.zeros((1, 2), dtype=np.uint32)
    wi, wm = np.empty(1, np.uint32), np.empty(1, np.float32)
    for a in range(len(sizes)):
        srv.wait(srv.submit(a, warm, wi, wm))  # every initial array built
    mark("register")
    with ClockSampler(dev.index) as clocks:
        lat, wall = srv.replay(ev, lr, out_i, out_m)
    st = srv.stats()
    lat_req = lat[req & (lat >= 0)]
    mark("replay")

    # parity: a sample of requests on the smaller arrays against the CPU oracle
    parity = True
    cand = [i for i in np.flatnonzero(req) if n_of[int(ev["array_id"][i])] <= (1 << 22)]
    for i in rng.choice(cand, size=min(len(cand), 6), replace=False):
        aid, o, q = int(ev["array_id"][i]), int(ev["q_offset"][i]), int(ev["q"][i])
        v = torch.empty(n_of[aid], dtype=torch.float32, device=dev)
        R.gen_values_device(v, seed_of(aid))
        x = v.cpu().numpy()
        parity &= np.array_equal(out_i[o:o + q], oracle.rmq_argmin(x, lr[o:o + q]))
        parity &= out_m[o:o + q].tobytes() == oracle.rmq_min(x, lr[o:o + q]).tobytes()

    mark("parity")
    # capacity: requests on the initial arrays, all issued at once
    cap_ev = ev[req & (ev["array_id"] < len(sizes))].copy()
    cap_ev["t_arrival_s"] = 0.0
    cap_q = int(cap_ev["q"].sum())
    _, cap_wall = srv.replay(cap_ev, lr, out_i, out_m)
    cap_stats = srv.stats()
    srv.close()
    mark("capacity")

    # the comparator: a C-side per-request loop of the plain kernel on
    # prebuilt handles, with page-locked host buffers (rmq_query_idx_host's
    # direct path: one launch per request, queries read from and results
    # written to host memory, waited for before the next request)
    vals, hs = [], []
    stream = torch.cuda.Stream(device=dev)
    for a, n in enumerate(sizes):
        v = torch.empty(n, dtype=torch.float32, device=dev)
        R.gen_values_device(v, seed_of(a))
        vals.append(v)
        hs.append(R.Hierarchy(v, variant="vl", t=64, stream=stream))
    h_i = torch.ones(Q, dtype=torch.int32).pin_memory()
    h_m = torch.ones(Q, dtype=torch.float32).pin_memory()
    torch.cuda.synchronize()
    mark("loop_setup")
    R.serve_serial_loop(hs, cap_ev[:64], lr_t, h_i, h_m)  # warm-up
    loop_s = R.serve_serial_loop(hs, cap_ev, lr_t, h_i, h_m)
    loop_same = True
    for e in cap_ev[:: max(1, cap_ev.size // 64)]:
        o, q = int(e["q_offset"]), int(e["q"])
        loop_same &= bool(np.array_equal(h_i[o:o + q].numpy().view(np.uint32), out_i[o:o + q]))
    for h in hs:
        h.close()
    del vals, h_i, h_m
    mark("loop")

    return {
        "metric": "RMQ queries/s (served: continuous batching)", "value": Q / wall, "unit": UNIT,
        "steps": 1, "warmup": 1, "ms_per_step": wall * 1e3,
        "workload": f"serving: {args.serve_arrays} resident arrays log-uniform [2^16, 2^{args.serve_max_log2:g}], "
                    "Poisson 20k req/s, 1..2^16 queries per request (log-uniform), lognormal(2^13, 1) lengths, "
                    f"5 % registrations, {args.serve_budget_gib:g} GiB budget, LRU eviction",
        "data": "synthetic (seeded Poisson trace)",
        "seconds": args.serve_seconds, "events": int(ev.size), "requests": int(req.sum()),
        "queries": Q, "slots": args.serve_slots, "seed": args.seed,
        "query_threads": args.serve_threads or "library default",
        "latency_us": {"p50": float(np.percentile(lat_req, 50)), "p99": float(np.percentile(lat_req, 99)),
                       "mean": float(lat_req.mean()), "max": float(lat_req.max())},
        "offered_queries_per_s": Q / float(ev["t_arrival_s"][-1]),
        "server_stats": st,
        "capacity": {"value": cap_q / cap_wall, "requests": int(cap_ev.size), "queries": cap_q,
                     "what": "same requests on the initial arrays, all arriving at once",
                     "batches": int(cap_stats["batches"] - st["batches"]),
                     "requests_answered_in_place": int(cap_stats["direct_requests"] - st["direct_requests"])},
        "request_buffers": "page-locked (queries read and results written in place by the batch kernel)",
        "phase_s": phase,
        "loop_plain_kernel": {"value": cap_q / loop_s, "seconds": loop_s, "results_equal_served": loop_same,
                              "what": "rmq_serve_serial_loop (C side): per request rmq_query_idx_host on a "
                                      "prebuilt handle, page-locked buffers, waited for before the next"},
        "speedup_capacity_vs_loop": (cap_q / cap_wall) / (cap_q / loop_s),
        "clocks": clocks.summary(), "parity_sample_ok": bool(parity),
    }


def run_serve(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    rec = served_record(args, ws, rank, torch.device("cuda", local))
    line = {"metric": rec.pop("metric"), "value": rec.pop("value"), "unit": rec.pop("unit"), "n_gpus": ws,
            "steps": 1, "warmup": 1, "ms_per_step": rec.pop("ms_per_step"), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": rec.pop("data"),
            "config": {"workload": rec.pop("workload"), "seconds": rec["seconds"], "events": rec["events"],
                       "requests": rec["requests"], "queries": rec["queries"], "slots": rec["slots"],
                       "seed": args.seed, "query_threads": rec["query_threads"]}}
    line.update(rec)
    if rank == 0:
        print(json.dumps(line), flush=True)


def parse_args(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--mode", choices=["plain", "batched", "serve"], default="plain",
                    help="plain = the single-array workload (default); batched = 4096 arrays; "
                         "serve = the request-serving loop")
    ap.add_argument("--sub-records", dest="sub_records", default="all",
                    help="plain mode: sub-records after the headline: all (default), none, or a comma list of "
                         + ", ".join(SUB_RECORDS))
    ap.add_argument("--serve-seconds", dest="serve_seconds", type=float, default=2.0)
    ap.add_argument("--serve-slots", dest="serve_slots", type=int, default=4)
    ap.add_argument("--serve-arrays", dest="serve_arrays", type=int, default=256,
                    help="initially resident arrays of the served workload (a smaller case for profiling)")
    ap.add_argument("--serve-max-log2", dest="serve_max_log2", type=float, default=26.0,
                    help="largest served array size, as log2 (sizes are log-uniform from 2^16)")
    ap.add_argument("--serve-budget-gib", dest="serve_budget_gib", type=float, default=64.0,
                    help="HBM budget of the server, GiB")
    ap.add_argument("--serve-threads", dest="serve_threads", type=int, default=0,
                    help="CTA size of the served query kernel (0 = library default)")
    ap.add_argument("--batch-arrays", dest="batch_arrays", type=int, default=4096)
    ap.add_argument("--n", type=int, default=1 << 26)
    ap.add_argument("--q", type=int, default=1 << 26)
    ap.add_argument("--lr", type=int, default=-7, help="length law code (-7 = lognormal median 2^13 sigma 1)")
    ap.add_argument("--seed", type=int, default=42)
    ap.add_argument("--ties", type=float, default=0.0,
                    help="fraction of entries set to the global minimum (the large mixed workload uses 0.01)")
    ap.add_argument("--variant", default="auto",
                    choices=["auto", "cl", "vl", "vl-short", "cl-noshuffle", "cl-tile", "cl-atomic"])
    ap.add_argument("--t", type=int, default=1 << 10, help="scan threshold")
    ap.add_argument("--rf-log", dest="rf_log", type=int, default=0)
    ap.add_argument("--lanes", type=int, default=0)
    ap.add_argument("--l2-persist", dest="l2_persist", action="store_true")
    ap.add_argument("--no-t-sweep", dest="t_sweep", action="store_false",
                    help="skip the scan-threshold sweep of the headline workload")
    ap.add_argument("--cpu-budget", dest="cpu_budget", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", dest="no_cpu_baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", dest="no_reference_gpu", action="store_true")
    ap.add_argument("--ref-step-queries", dest="ref_step_queries", type=int, default=1 << 14)
    args = ap.parse_args(argv)
    args.warmup = max(3, args.warmup)  # timing rule: at least 3 untimed warm-up steps
    return args


def main(argv=None):
    args = parse_args(argv)
    ws, rank, local = dist_env()
    if args.gpus != ws and rank == 0:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={ws}; one process per GPU is started by "
              f"torchrun, and the line reports the {ws} rank(s) that run", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.mode == "batched":
        run_batched(args, ws, rank, local)
        return
    if args.mode == "serve":
        run_serve(args, ws, rank, local)
        return
    run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
