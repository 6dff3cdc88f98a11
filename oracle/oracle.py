"""ctypes loader for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and the CPU legs of bench.py import this
module, and only as the checker or as the timed CPU baseline.

  liboracle.so        restatement of the reference's brute-force scan
                      (src/cpu_methods.h:7-77) plus a sparse-table oracle and
                      the level-layout rule (src/xxx.h:225-243), rmq_oracle.c;
                      and of its input generators (src/rand.cuh:49-240),
                      rmq_oracle_gen.cpp
  _ref/librmq_ref.so  the reference's own generator and CPU scan, compiled from
                      its sources by build_ref.sh where they are present
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "librmq_ref.so"

_P = ctypes.c_void_p
_U64 = ctypes.c_uint64
_o = None
_r = None


def lib() -> ctypes.CDLL:
    global _o
    if _o is None:
        if not ORACLE_LIB.exists():
            raise RuntimeError(f"{ORACLE_LIB} missing: run the build first")
        L = ctypes.CDLL(str(ORACLE_LIB))
        L.oracle_min.argtypes = [_P, _U64, _P, _U64, _P, ctypes.c_int]
        L.oracle_argmin.argtypes = [_P, _U64, _P, _U64, _P, ctypes.c_int]
        L.oracle_max_threads.restype = ctypes.c_int
        L.oracle_sparse_build.argtypes = [_P, _U64]
        L.oracle_sparse_build.restype = _P
        L.oracle_sparse_free.argtypes = [_P]
        L.oracle_sparse_query.argtypes = [_P, _P, _U64, _P, _P, ctypes.c_int]
        L.oracle_layout.argtypes = [_U64, _U64, ctypes.c_int, _P, _P, _P]
        L.oracle_cpu_rmq.argtypes = [_P, _P, _U64, _P, ctypes.c_int]
        L.oracle_cpu_rmq_idx.argtypes = [_P, _P, _U64, _P, ctypes.c_int]
        L.oracle_gen_array.argtypes = [_U64, ctypes.c_int32, _P]
        L.oracle_gen_queries.argtypes = [_U64, ctypes.c_int32, _U64, ctypes.c_int32, _P]
        L.oracle_gen_queries.restype = ctypes.c_int32
        L.oracle_plant_min_ties.argtypes = [_P, _U64, ctypes.c_double, ctypes.c_int32]
        _o = L
    return _o


def ref_available() -> bool:
    return REF_LIB.exists()


def ref() -> ctypes.CDLL:
    global _r
    if _r is None:
        R = ctypes.CDLL(str(REF_LIB))
        R.ref_random_array.argtypes = [ctypes.c_uint32, ctypes.c_int, _P]
        R.ref_random_queries.argtypes = [ctypes.c_uint32, ctypes.c_int, ctypes.c_uint32, ctypes.c_int,
                                         ctypes.c_int, _P]
        R.ref_sample_indices.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, _P]
        R.ref_sample_indices.restype = ctypes.c_uint32
        R.ref_cpu_rmq.argtypes = [ctypes.c_uint32, ctypes.c_uint32, _P, _P, ctypes.c_int, _P]
        R.ref_cpu_rmq_idx.argtypes = [ctypes.c_uint32, ctypes.c_uint32, _P, _P, ctypes.c_int, _P]
        _r = R
    return _r


def _c(a: np.ndarray) -> int:
    assert a.flags.c_contiguous
    return a.ctypes.data


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def rmq_min(a: np.ndarray, qs: np.ndarray, nthreads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    qs = np.ascontiguousarray(qs, dtype=np.uint32)
    q = qs.size // 2
    out = np.empty(q, dtype=np.float32)
    lib().oracle_min(_c(a), a.size, _c(qs), q, _c(out), nthreads)
    return out


def rmq_argmin(a: np.ndarray, qs: np.ndarray, nthreads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    qs = np.ascontiguousarray(qs, dtype=np.uint32)
    q = qs.size // 2
    out = np.empty(q, dtype=np.uint32)
    lib().oracle_argmin(_c(a), a.size, _c(qs), q, _c(out), nthreads)
    return out


def cpu_rmq(a: np.ndarray, qs: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """cpu_rmq as the reference runs it (default OpenMP schedule); valid
    queries only.  The timed CPU baseline."""
    q = qs.size // 2
    out = np.empty(q, dtype=np.float32)
    lib().oracle_cpu_rmq(_c(a), _c(qs), q, _c(out), nthreads)
    return out


def cpu_rmq_idx(a: np.ndarray, qs: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """cpu_rmq_idx as the reference runs it; valid queries only."""
    q = qs.size // 2
    out = np.empty(q, dtype=np.uint32)
    lib().oracle_cpu_rmq_idx(_c(a), _c(qs), q, _c(out), nthreads)
    return out


def gen_array(n: int, seed: int) -> np.ndarray:
    """The reference's random_array_par_cpu (src/rand.cuh:49-61)."""
    a = np.empty(n, dtype=np.float32)
    lib().oracle_gen_array(n, seed, _c(a))
    return a


def gen_queries(q: int, lr: int, n: int, seed: int) -> np.ndarray:
    """The reference's random_queries_par_cpu (src/rand.cuh:181-217) and the
    added laws -7 / -8, as inclusive [q, 2] uint32 pairs."""
    out = np.empty((q, 2), dtype=np.uint32)
    if lib().oracle_gen_queries(q, lr, n, seed, _c(out)) != 0:
        raise ValueError(f"unknown length law lr={lr} for n={n}")
    return out


def plant_min_ties(a: np.ndarray, frac: float, seed: int) -> np.ndarray:
    lib().oracle_plant_min_ties(_c(a), a.size, frac, seed)
    return a


class Sparse:
    """Fast oracle: block minima + sparse table, (value, index) order."""

    def __init__(self, a: np.ndarray):
        self.a = np.ascontiguousarray(a, dtype=np.float32)
        self.h = lib().oracle_sparse_build(_c(self.a), self.a.size)
        if not self.h:
            raise MemoryError("oracle_sparse_build failed")

    def query(self, qs: np.ndarray, nthreads: int = 0):
        qs = np.ascontiguousarray(qs, dtype=np.uint32)
        q = qs.size // 2
        m = np.empty(q, dtype=np.float32)
        i = np.empty(q, dtype=np.uint32)
        lib().oracle_sparse_query(self.h, _c(qs), q, _c(m), _c(i), nthreads)
        return m, i

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_sparse_free(self.h)
            self.h = None


def layout(n: int, t: int, rf_log: int):
    sizes = np.zeros(20, dtype=np.uint64)
    offs = np.zeros(20, dtype=np.uint64)
    nl = np.zeros(1, dtype=np.uint32)
    lib().oracle_layout(n, t, rf_log, _c(nl), _c(sizes), _c(offs))
    k = int(nl[0])
    return k, [int(x) for x in sizes[:k]], [int(x) for x in offs[:k]]


# ---- reference build (pinning) ------------------------------------------------

def ref_array(n: int, seed: int) -> np.ndarray:
    a = np.empty(n, dtype=np.float32)
    ref().ref_random_array(n, seed, _c(a))
    return a


def ref_queries(q: int, lr: int, n: int, seed: int, trivial: bool = False) -> np.ndarray:
    out = np.empty((q, 2), dtype=np.uint32)
    ref().ref_random_queries(q, lr, n, seed, 1 if trivial else 0, _c(out))
    return out


def ref_min(a: np.ndarray, qs: np.ndarray, nthreads: int = 4) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    qs = np.ascontiguousarray(qs, dtype=np.uint32)
    q = qs.size // 2
    out = np.empty(q, dtype=np.float32)
    ref().ref_cpu_rmq(a.size, q, _c(a), _c(qs), nthreads, _c(out))
    return out


def ref_argmin(a: np.ndarray, qs: np.ndarray, nthreads: int = 4) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    qs = np.ascontiguousarray(qs, dtype=np.uint32)
    q = qs.size // 2
    out = np.empty(q, dtype=np.uint32)
    ref().ref_cpu_rmq_idx(a.size, q, _c(a), _c(qs), nthreads, _c(out))
    return out


def ref_sample_indices(original: int, sample: int, seed: int) -> np.ndarray:
    out = np.empty(min(original, sample), dtype=np.uint32)
    m = ref().ref_sample_indices(original, sample, seed, _c(out))
    return out[:m]
