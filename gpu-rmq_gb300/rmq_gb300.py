"""Python binding of the GB300 RMQ C ABI (include/rmq_gb300.h) over ctypes.

This is the host-side mirror used by the tests and bench.py.  The work is done
by librmq_gb300.so (hand-written CUDA for sm_103a); this module only moves
pointers and sizes across the C boundary.  There is no fallback: if the
library is missing, every entry point raises.

Reference mapping (reference files, by path within the reference project):
  Hierarchy(...).query      xxx_rmq / hierarchical_vector_load (src/xxx.h:204, :933)
  Hierarchy(...).query_idx  argmin over the hierarchy (new; results of
                            gpu_rmq_basic_idx, src/cuda_methods.cuh:106)
  bruteforce(...)           gpu_rmq_basic{,_idx} (src/cuda_methods.cuh:72-137)
  gen_array / gen_queries   random_array_par_cpu / random_queries_par_cpu
                            (src/rand.cuh:49-217)
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
# RMQ_GB300_LIB overrides the library path (e.g. an alternative build of the
# same sources); the default is the in-tree build.
LIB_PATH = Path(os.environ.get("RMQ_GB300_LIB", str(PKG / "librmq_gb300.so")))
GEN_PATH = PKG / "librmq_gen.so"

RMQ_OK = 0
RMQ_ERR_ARG = 1
RMQ_ERR_CUDA = 2
RMQ_ERR_OOM = 3
RMQ_ERR_QUERY_RANGE = 4
RMQ_ERR_TIMEOUT = 5
RMQ_ERR_NO_INDEX = 6
RMQ_ERR_UNSUPPORTED = 7

VARIANT_AUTO = 0
VARIANT_CL = 1
VARIANT_VL = 2
VARIANT_CL_NO_SHUFFLE = 3      # the reference's ablations of CL (algs 23, 24, 19)
VARIANT_CL_QUERY_PER_TILE = 4
VARIANT_CL_ATOMIC = 5
VARIANT_VL_SHORT = 6           # VL for workloads of short queries
VARIANTS = {"auto": VARIANT_AUTO, "cl": VARIANT_CL, "vl": VARIANT_VL, "cl-noshuffle": VARIANT_CL_NO_SHUFFLE,
            "cl-tile": VARIANT_CL_QUERY_PER_TILE, "cl-atomic": VARIANT_CL_ATOMIC, "vl-short": VARIANT_VL_SHORT}

NO_POS = 0xFFFFFFFF


class RMQConfig(ctypes.Structure):
    _fields_ = [
        ("variant", ctypes.c_int32),
        ("scan_threshold", ctypes.c_uint64),
        ("rf_log", ctypes.c_int32),
        ("lanes", ctypes.c_int32),
        ("with_index", ctypes.c_int32),
        ("l2_persist", ctypes.c_int32),
        ("validate", ctypes.c_int32),
        ("index_bits", ctypes.c_int32),
    ]


class RMQInfo(ctypes.Structure):
    _fields_ = [
        ("num_levels", ctypes.c_uint32),
        ("rf_log", ctypes.c_uint32),
        ("variant", ctypes.c_int32),
        ("lanes", ctypes.c_int32),
        ("n", ctypes.c_uint64),
        ("scan_threshold", ctypes.c_uint64),
        ("level_size", ctypes.c_uint64 * 20),
        ("level_offset", ctypes.c_uint64 * 20),
        ("level_bytes", ctypes.c_uint64),
        ("build_ms", ctypes.c_float),
        ("index_bits", ctypes.c_int32),
    ]

    def sizes(self) -> list[int]:
        return [int(self.level_size[k]) for k in range(self.num_levels)]

    def offsets(self) -> list[int]:
        return [int(self.level_offset[k]) for k in range(self.num_levels)]


class RMQError(RuntimeError):
    def __init__(self, status: int, what: str):
        self.status = status
        super().__init__(f"{what}: {strerror(status)} (status {status})")


_lib = None
_gen = None

_P = ctypes.c_void_p
_U64 = ctypes.c_uint64


def lib() -> ctypes.CDLL:
    """Loads librmq_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"`")
        L = ctypes.CDLL(str(LIB_PATH))
        L.rmq_config_init.argtypes = [ctypes.POINTER(RMQConfig)]
        L.rmq_config_init.restype = None
        L.rmq_build.argtypes = [_P, _U64, ctypes.POINTER(RMQConfig), _P, ctypes.POINTER(_P)]
        L.rmq_build.restype = ctypes.c_int
        L.rmq_query.argtypes = [_P, _P, _U64, _P, _P]
        L.rmq_query.restype = ctypes.c_int
        L.rmq_query_idx.argtypes = [_P, _P, _U64, _P, _P, _P]
        L.rmq_query_idx.restype = ctypes.c_int
        L.rmq_query64.argtypes = [_P, _P, _U64, _P, _P]
        L.rmq_query64.restype = ctypes.c_int
        L.rmq_query_idx64.argtypes = [_P, _P, _U64, _P, _P, _P]
        L.rmq_query_idx64.restype = ctypes.c_int
        L.rmq_query_host.argtypes = [_P, _P, _U64, _P]
        L.rmq_query_host.restype = ctypes.c_int
        L.rmq_query_idx_host.argtypes = [_P, _P, _U64, _P, _P]
        L.rmq_query_idx_host.restype = ctypes.c_int
        L.rmq_query64_host.argtypes = [_P, _P, _U64, _P]
        L.rmq_query64_host.restype = ctypes.c_int
        L.rmq_query_idx64_host.argtypes = [_P, _P, _U64, _P, _P]
        L.rmq_query_idx64_host.restype = ctypes.c_int
        L.rmq_scan_bruteforce.argtypes = [_P, _U64, _P, _U64, _P, _P, _P]
        L.rmq_scan_bruteforce.restype = ctypes.c_int
        L.rmq_get_info.argtypes = [_P, ctypes.POINTER(RMQInfo)]
        L.rmq_get_info.restype = ctypes.c_int
        L.rmq_destroy.argtypes = [_P]
        L.rmq_destroy.restype = None
        L.rmq_strerror.argtypes = [ctypes.c_int]
        L.rmq_strerror.restype = ctypes.c_char_p
        L.rmq_debug_bounds_violations.argtypes = [ctypes.POINTER(_U64)]
        L.rmq_debug_bounds_violations.restype = ctypes.c_int
        L.rmq_plan_layout.argtypes = [_U64, _U64, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(RMQInfo)]
        L.rmq_plan_layout.restype = ctypes.c_int
        L.rmq_measure_l2_read.argtypes = [_P, _U64, ctypes.c_uint32, ctypes.c_int32, _P,
                                          ctypes.POINTER(ctypes.c_float)]
        L.rmq_measure_l2_read.restype = ctypes.c_int
        _lib = L
    return _lib


def genlib() -> ctypes.CDLL:
    global _gen
    if _gen is None:
        if not GEN_PATH.exists():
            raise RuntimeError(f"{GEN_PATH} is missing: build the package first")
        G = ctypes.CDLL(str(GEN_PATH))
        G.rmq_gen_array.argtypes = [_U64, ctypes.c_int32, _P]
        G.rmq_gen_array.restype = None
        G.rmq_gen_queries.argtypes = [_U64, ctypes.c_int32, _U64, ctypes.c_int32, ctypes.c_int32, _P]
        G.rmq_gen_queries.restype = ctypes.c_int32
        G.rmq_gen_plant_min_ties.argtypes = [_P, _U64, ctypes.c_double, ctypes.c_int32]
        G.rmq_gen_plant_min_ties.restype = None
        G.rmq_gen_sample_indices.argtypes = [_U64, _U64, ctypes.c_int32, _P]
        G.rmq_gen_sample_indices.restype = _U64
        _gen = G
    return _gen


def strerror(status: int) -> str:
    return lib().rmq_strerror(status).decode()


def config(variant: str | int = "auto", t: int = 0, rf_log: int = 0, lanes: int = 0,
           with_index: bool = True, l2_persist: bool = False, validate: bool = False,
           index_bits: int = 0) -> RMQConfig:
    cfg = RMQConfig()
    lib().rmq_config_init(ctypes.byref(cfg))
    cfg.variant = VARIANTS[variant] if isinstance(variant, str) else int(variant)
    cfg.scan_threshold = int(t)
    cfg.rf_log = int(rf_log)
    cfg.lanes = int(lanes)
    cfg.with_index = 1 if with_index else 0
    cfg.l2_persist = 1 if l2_persist else 0
    cfg.validate = 1 if validate else 0
    cfg.index_bits = int(index_bits)
    return cfg


def plan_layout(n: int, t: int = 0, rf_log: int = 0, variant: str | int = "auto") -> RMQInfo:
    """Level layout for n entries (host-only, no GPU needed)."""
    info = RMQInfo()
    v = VARIANTS[variant] if isinstance(variant, str) else int(variant)
    st = lib().rmq_plan_layout(n, t, rf_log, v, ctypes.byref(info))
    if st != RMQ_OK:
        raise RMQError(st, "rmq_plan_layout")
    return info


def measure_l2_read(buf, passes: int = 20, random: bool = False, stream=None) -> float:
    """L2-resident sector read rate in GB/s over a CUDA float32 tensor (its
    byte size / 32 a power of two; values >= -1) that fits in L2."""
    ms = ctypes.c_float()
    nbytes = buf.numel() * 4
    st = lib().rmq_measure_l2_read(_dev_ptr(buf), nbytes, passes, 1 if random else 0,
                                   _stream_handle(stream), ctypes.byref(ms))
    if st != RMQ_OK:
        raise RMQError(st, "rmq_measure_l2_read")
    return nbytes * passes / (ms.value / 1e3) / 1e9


def _stream_handle(stream) -> int:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _dev_ptr(t) -> int:
    return int(t.data_ptr())


class Hierarchy:
    """A built hierarchy over a device-resident float32 tensor (torch)."""

    def __init__(self, values, variant: str | int = "auto", t: int = 0, rf_log: int = 0,
                 lanes: int = 0, with_index: bool = True, l2_persist: bool = False,
                 validate: bool = False, stream=None, index_bits: int = 0):
        import torch
        if not isinstance(values, torch.Tensor) or values.device.type != "cuda":
            raise TypeError("values must be a CUDA torch tensor")
        if values.dtype != torch.float32 or not values.is_contiguous():
            raise TypeError("values must be contiguous float32")
        self.values = values  # level 0 is the caller's array: keep it alive
        self.n = values.numel()
        cfg = config(variant, t, rf_log, lanes, with_index, l2_persist, validate, index_bits)
        h = _P()
        st = lib().rmq_build(_dev_ptr(values), self.n, ctypes.byref(cfg), _stream_handle(stream),
                             ctypes.byref(h))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_build")
        self._h = h

    @property
    def handle(self) -> int:
        return self._h.value

    def info(self) -> RMQInfo:
        info = RMQInfo()
        st = lib().rmq_get_info(self._h, ctypes.byref(info))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_get_info")
        return info

    def query_raw(self, lr_ptr: int, q: int, out_min_ptr: int, stream=None) -> int:
        return lib().rmq_query(self._h, lr_ptr, q, out_min_ptr, _stream_handle(stream))

    def query_idx_raw(self, lr_ptr: int, q: int, out_idx_ptr: int, out_min_ptr: int | None,
                      stream=None) -> int:
        return lib().rmq_query_idx(self._h, lr_ptr, q, out_idx_ptr, out_min_ptr or None,
                                   _stream_handle(stream))

    def query(self, lr, out=None, stream=None):
        """Minima of the inclusive queries in lr (CUDA uint32/int32 tensor, shape [q, 2])."""
        import torch
        q = lr.numel() // 2
        if out is None:
            out = torch.empty(q, dtype=torch.float32, device=lr.device)
        st = self.query_raw(_dev_ptr(lr), q, _dev_ptr(out), stream)
        if st != RMQ_OK:
            raise RMQError(st, "rmq_query")
        return out

    def query_idx(self, lr, out_idx=None, out_min=None, with_min: bool = False, stream=None):
        import torch
        q = lr.numel() // 2
        if out_idx is None:
            out_idx = torch.empty(q, dtype=torch.int32, device=lr.device)
        if with_min and out_min is None:
            out_min = torch.empty(q, dtype=torch.float32, device=lr.device)
        st = self.query_idx_raw(_dev_ptr(lr), q, _dev_ptr(out_idx),
                                _dev_ptr(out_min) if out_min is not None else None, stream)
        if st != RMQ_OK:
            raise RMQError(st, "rmq_query_idx")
        return (out_idx, out_min) if with_min else out_idx

    def query64(self, lr, out=None, stream=None):
        """Minima of 64-bit inclusive queries (CUDA int64 tensor [q, 2]); 64-bit handles."""
        import torch
        q = lr.numel() // 2
        if out is None:
            out = torch.empty(q, dtype=torch.float32, device=lr.device)
        st = lib().rmq_query64(self._h, _dev_ptr(lr), q, _dev_ptr(out), _stream_handle(stream))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_query64")
        return out

    def query_idx64(self, lr, with_min: bool = False, stream=None):
        """Argmin (int64 tensor) and optionally minima of 64-bit queries."""
        import torch
        q = lr.numel() // 2
        out_idx = torch.empty(q, dtype=torch.int64, device=lr.device)
        out_min = torch.empty(q, dtype=torch.float32, device=lr.device) if with_min else None
        st = lib().rmq_query_idx64(self._h, _dev_ptr(lr), q, _dev_ptr(out_idx),
                                   _dev_ptr(out_min) if out_min is not None else None, _stream_handle(stream))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_query_idx64")
        return (out_idx, out_min) if with_min else out_idx

    def query_idx_host_raw(self, lr_ptr: int, q: int, out_idx_ptr: int, out_min_ptr: int | None) -> int:
        """rmq_query_idx_host on host pointers (blocking)."""
        return lib().rmq_query_idx_host(self._h, lr_ptr, q, out_idx_ptr, out_min_ptr or None)

    def query_host(self, lr: np.ndarray) -> np.ndarray:
        """Minima of host queries (numpy [q, 2] uint32 or uint64) into a host array."""
        lr = np.ascontiguousarray(lr)
        q = lr.shape[0]
        out = np.empty(q, dtype=np.float32)
        wide = lr.dtype.itemsize == 8
        fn = lib().rmq_query64_host if wide else lib().rmq_query_host
        st = fn(self._h, lr.ctypes.data, q, out.ctypes.data)
        if st != RMQ_OK:
            raise RMQError(st, "rmq_query64_host" if wide else "rmq_query_host")
        return out

    def query_idx_host(self, lr: np.ndarray, with_min: bool = False):
        """Argmin (and optionally minima) of host queries into host arrays."""
        lr = np.ascontiguousarray(lr)
        q = lr.shape[0]
        wide = lr.dtype.itemsize == 8
        out_idx = np.empty(q, dtype=np.uint64 if wide else np.uint32)
        out_min = np.empty(q, dtype=np.float32) if with_min else None
        fn = lib().rmq_query_idx64_host if wide else lib().rmq_query_idx_host
        st = fn(self._h, lr.ctypes.data, q, out_idx.ctypes.data,
                out_min.ctypes.data if out_min is not None else None)
        if st != RMQ_OK:
            raise RMQError(st, "rmq_query_idx64_host" if wide else "rmq_query_idx_host")
        return (out_idx, out_min) if with_min else out_idx

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            lib().rmq_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def bruteforce(values, lr, want_min: bool = True, want_idx: bool = True, stream=None):
    """The GPU brute-force checker (one warp per query)."""
    import torch
    q = lr.numel() // 2
    out_min = torch.empty(q, dtype=torch.float32, device=lr.device) if want_min else None
    out_idx = torch.empty(q, dtype=torch.int32, device=lr.device) if want_idx else None
    st = lib().rmq_scan_bruteforce(_dev_ptr(values), values.numel(), _dev_ptr(lr), q,
                                   _dev_ptr(out_min) if out_min is not None else None,
                                   _dev_ptr(out_idx) if out_idx is not None else None,
                                   _stream_handle(stream))
    if st != RMQ_OK:
        raise RMQError(st, "rmq_scan_bruteforce")
    return out_min, out_idx


# ---- host generators (librmq_gen.so) ----------------------------------------

def gen_array(n: int, seed: int) -> np.ndarray:
    a = np.empty(n, dtype=np.float32)
    genlib().rmq_gen_array(n, seed, a.ctypes.data)
    return a


def gen_queries(q: int, lr: int, n: int, seed: int, trivial: bool = False) -> np.ndarray:
    out = np.empty((q, 2), dtype=np.uint32)
    rc = genlib().rmq_gen_queries(q, lr, n, seed, 1 if trivial else 0, out.ctypes.data)
    if rc != 0:
        raise ValueError(f"unknown length law lr={lr} for n={n}")
    return out


def plant_min_ties(a: np.ndarray, frac: float, seed: int) -> np.ndarray:
    genlib().rmq_gen_plant_min_ties(a.ctypes.data, a.size, frac, seed)
    return a


def sample_indices(original_size: int, sample_size: int, seed: int) -> np.ndarray:
    out = np.empty(min(original_size, sample_size), dtype=np.uint32)
    m = genlib().rmq_gen_sample_indices(original_size, sample_size, seed, out.ctypes.data)
    return out[:m]


# ---- batched queries over many arrays (include/rmq_gb300_batch.h) ------------

class BatchInfo(ctypes.Structure):
    _fields_ = [
        ("num_arrays", ctypes.c_uint32),
        ("total_values", ctypes.c_uint64),
        ("level_bytes", ctypes.c_uint64),
        ("scan_threshold", ctypes.c_uint64),
        ("query_block", ctypes.c_uint32),
        ("max_levels", ctypes.c_uint32),
        ("total_queries", ctypes.c_uint64),
        ("build_ms", ctypes.c_float),
        ("query_ms", ctypes.c_float),
        ("class_threshold", ctypes.c_uint64 * 3),
        ("class_upper", ctypes.c_uint64 * 3),
    ]


_batch_bound = False


def _bind_batch() -> ctypes.CDLL:
    global _batch_bound
    L = lib()
    if not _batch_bound:
        L.rmq_batch_create.argtypes = [_P, _P, _P, ctypes.c_uint32, ctypes.POINTER(RMQConfig), _P,
                                       ctypes.POINTER(_P)]
        L.rmq_batch_set_queries.argtypes = [_P, _P, _P, _P, _P, _P]
        for name in ("rmq_batch_build", "rmq_batch_query", "rmq_batch_run", "rmq_batch_run_per_array"):
            getattr(L, name).argtypes = [_P, _P]
        L.rmq_batch_autotune.argtypes = [_P, _P, ctypes.POINTER(BatchInfo)]
        L.rmq_batch_get_info.argtypes = [_P, ctypes.POINTER(BatchInfo)]
        L.rmq_batch_set_tuning.argtypes = [_P, _U64, ctypes.c_uint32, _P]
        L.rmq_batch_set_class_tuning.argtypes = [_P, _P, ctypes.c_uint32, _P]
        L.rmq_batch_destroy.argtypes = [_P]
        L.rmq_batch_destroy.restype = None
        L.rmq_gen_values_device.argtypes = [_P, _U64, _U64, _P]
        L.rmq_gen_queries_device.argtypes = [_P, _U64, _U64, ctypes.c_int32, ctypes.c_double,
                                             ctypes.c_double, _U64, _P]
        _batch_bound = True
    return L


class Batch:
    """Many independent arrays packed in one device tensor; one build pass and
    one query launch (or one graph launch) for all of them."""

    def __init__(self, values, value_offsets, sizes, t: int = 0, with_index: bool = True, stream=None):
        L = _bind_batch()
        self.values = values
        self.offsets = np.ascontiguousarray(value_offsets, dtype=np.uint64)
        self.sizes = np.ascontiguousarray(sizes, dtype=np.uint64)
        self.num_arrays = int(self.sizes.size)
        cfg = config("vl", t, 3, 0, with_index)
        h = _P()
        st = L.rmq_batch_create(_dev_ptr(values), self.offsets.ctypes.data, self.sizes.ctypes.data,
                                self.num_arrays, ctypes.byref(cfg), _stream_handle(stream), ctypes.byref(h))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_batch_create")
        self._h = h
        self._keep = ()

    def set_queries(self, lr, query_offsets, out_idx=None, out_min=None, stream=None):
        qo = np.ascontiguousarray(query_offsets, dtype=np.uint64)
        self._keep = (lr, out_idx, out_min, qo)
        self.query_offsets = qo
        st = _bind_batch().rmq_batch_set_queries(
            self._h, _dev_ptr(lr) if lr.numel() else None, qo.ctypes.data,
            _dev_ptr(out_idx) if out_idx is not None else None,
            _dev_ptr(out_min) if out_min is not None else None, _stream_handle(stream))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_batch_set_queries")

    def _call(self, name, stream):
        st = getattr(_bind_batch(), name)(self._h, _stream_handle(stream))
        if st != RMQ_OK:
            raise RMQError(st, name)

    def build(self, stream=None):
        self._call("rmq_batch_build", stream)

    def query(self, stream=None):
        self._call("rmq_batch_query", stream)

    def run(self, stream=None):
        self._call("rmq_batch_run", stream)

    def run_per_array(self, stream=None):
        """The per-array loop of the plain kernels over the batch's buffers
        (the batched form's comparator; same results)."""
        self._call("rmq_batch_run_per_array", stream)

    def set_tuning(self, t: int, query_block: int, stream=None) -> None:
        """Applies a known (t, CTA size); rebuild before querying."""
        st = _bind_batch().rmq_batch_set_tuning(self._h, int(t), int(query_block), _stream_handle(stream))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_batch_set_tuning")

    def set_class_tuning(self, class_thresholds, query_block: int, stream=None) -> None:
        """Applies one t per array-size class (three values, as
        BatchInfo.class_threshold reports them); rebuild before querying."""
        arr = (ctypes.c_uint64 * 3)(*[int(x) for x in class_thresholds])
        st = _bind_batch().rmq_batch_set_class_tuning(self._h, arr, int(query_block), _stream_handle(stream))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_batch_set_class_tuning")

    def workload_key(self) -> str:
        """Identifies the tuning problem: the GPU, the array sizes and the
        per-array query counts (the autotuner times exactly these)."""
        import hashlib
        import torch
        hsh = hashlib.sha256()
        hsh.update(torch.cuda.get_device_name(self.values.device).encode())
        hsh.update(self.sizes.tobytes())
        hsh.update(np.diff(getattr(self, "query_offsets", np.zeros(1, np.uint64))).astype(np.uint64).tobytes())
        return hsh.hexdigest()[:32]

    def autotune(self, stream=None, cache: str | os.PathLike | None = None) -> BatchInfo:
        """Runs the autotuner, or, when `cache` (a JSON file) already holds a
        choice for this workload (workload_key), applies it and rebuilds.  A
        fresh choice is added to the cache."""
        import json
        key = self.workload_key() if cache is not None else None
        table = {}
        if cache is not None and Path(cache).exists():
            table = json.loads(Path(cache).read_text())
            hit = table.get(key)
            if hit is not None:
                if "class_threshold" in hit:
                    self.set_class_tuning(hit["class_threshold"], hit["query_block"], stream)
                else:
                    self.set_tuning(hit["scan_threshold"], hit["query_block"], stream)
                self.build(stream)
                return self.info()
        info = BatchInfo()
        st = _bind_batch().rmq_batch_autotune(self._h, _stream_handle(stream), ctypes.byref(info))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_batch_autotune")
        if cache is not None:
            table[key] = {"scan_threshold": int(info.scan_threshold), "query_block": int(info.query_block),
                          "class_threshold": [int(x) for x in info.class_threshold],
                          "query_ms": float(info.query_ms), "arrays": self.num_arrays}
            Path(cache).write_text(json.dumps(table, indent=1, sort_keys=True))
        return info

    def info(self) -> BatchInfo:
        info = BatchInfo()
        st = _bind_batch().rmq_batch_get_info(self._h, ctypes.byref(info))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_batch_get_info")
        return info

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _bind_batch().rmq_batch_destroy(self._h)
            self._h = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def gen_values_device(out, seed: int, stream=None):
    """Fills a CUDA float32 tensor with seeded uniform [0, 1) values."""
    st = _bind_batch().rmq_gen_values_device(_dev_ptr(out), out.numel(), seed, _stream_handle(stream))
    if st != RMQ_OK:
        raise RMQError(st, "rmq_gen_values_device")
    return out


def gen_queries_device(out, n: int, law: int, median: float = 1.0, sigma: float = 0.0, seed: int = 0,
                       stream=None):
    """Fills a CUDA int32 tensor of shape [q, 2] with seeded inclusive queries
    over n entries (law 0 = uniform length, 1 = lognormal(median, sigma))."""
    st = _bind_batch().rmq_gen_queries_device(_dev_ptr(out), out.numel() // 2, n, law, median, sigma, seed,
                                              _stream_handle(stream))
    if st != RMQ_OK:
        raise RMQError(st, "rmq_gen_queries_device")
    return out


def pack_offsets(sizes, align: int = 8) -> tuple[np.ndarray, int]:
    """Packed offsets of arrays laid end to end, each start a multiple of
    `align` entries (32 bytes for fp32 at align = 8); returns (offsets, total)."""
    sizes = np.asarray(sizes, dtype=np.uint64)
    padded = (sizes + np.uint64(align - 1)) // np.uint64(align) * np.uint64(align)
    offs = np.zeros(sizes.size, dtype=np.uint64)
    if sizes.size > 1:
        offs[1:] = np.cumsum(padded)[:-1]
    return offs, int(padded.sum())


# ---- the query server (include/rmq_gb300_serve.h) ----------------------------

class ServerConfig(ctypes.Structure):
    _fields_ = [
        ("hbm_budget_bytes", ctypes.c_uint64),
        ("slots", ctypes.c_uint32),
        ("max_batch_queries", ctypes.c_uint64),
        ("max_batch_requests", ctypes.c_uint32),
        ("scan_threshold", ctypes.c_uint64),
        ("query_threads", ctypes.c_uint32),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [(name, ctypes.c_uint64) for name in (
        "requests_done", "queries_done", "batches", "registrations", "evictions", "readmissions",
        "resident_arrays", "resident_bytes", "max_requests_per_batch", "max_batches_in_flight",
        "direct_requests")]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


# rmq_trace_event as a numpy record (C layout: double, int32 + 4 padding, 5 x uint64)
TRACE_DTYPE = np.dtype([("t_arrival_s", "<f8"), ("kind", "<i4"), ("_pad", "<i4"), ("array_id", "<u8"),
                        ("n", "<u8"), ("seed", "<u8"), ("q_offset", "<u8"), ("q", "<u8")])

_server_bound = False


def _bind_server() -> ctypes.CDLL:
    global _server_bound
    L = lib()
    if not _server_bound:
        L.rmq_server_config_init.argtypes = [ctypes.POINTER(ServerConfig)]
        L.rmq_server_config_init.restype = None
        L.rmq_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(_P)]
        L.rmq_server_register_generated.argtypes = [_P, _U64, _U64, ctypes.POINTER(_U64)]
        L.rmq_server_register_host.argtypes = [_P, _P, _U64, ctypes.POINTER(_U64)]
        L.rmq_server_submit.argtypes = [_P, _U64, _P, _U64, _P, _P, ctypes.POINTER(_U64)]
        L.rmq_server_wait.argtypes = [_P, _U64, ctypes.c_int64, ctypes.POINTER(ctypes.c_double)]
        L.rmq_server_drain.argtypes = [_P, ctypes.c_int64]
        L.rmq_server_replay.argtypes = [_P, _P, _U64, _P, _P, _P, _P, ctypes.POINTER(ctypes.c_double)]
        L.rmq_server_get_stats.argtypes = [_P, ctypes.POINTER(ServerStats)]
        L.rmq_server_fail_next_batches.argtypes = [_P, ctypes.c_uint32]
        L.rmq_serve_serial_loop.argtypes = [_P, _U64, _P, _U64, _P, _P, _P, ctypes.POINTER(ctypes.c_double)]
        L.rmq_server_destroy.argtypes = [_P]
        L.rmq_server_destroy.restype = None
        _server_bound = True
    return L


class Server:
    """Resident-array RMQ server with continuous batching (host buffers in/out)."""

    def __init__(self, hbm_budget_bytes: int = 0, slots: int = 0, max_batch_queries: int = 0,
                 max_batch_requests: int = 0, t: int = 0, query_threads: int = 0):
        L = _bind_server()
        cfg = ServerConfig()
        L.rmq_server_config_init(ctypes.byref(cfg))
        for name, val in (("hbm_budget_bytes", hbm_budget_bytes), ("slots", slots),
                          ("max_batch_queries", max_batch_queries), ("max_batch_requests", max_batch_requests),
                          ("scan_threshold", t), ("query_threads", query_threads)):
            if val:
                setattr(cfg, name, val)
        h = _P()
        st = L.rmq_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_server_create")
        self._h = h
        self._keep = {}

    def register_generated(self, n: int, seed: int) -> int:
        out = _U64()
        st = _bind_server().rmq_server_register_generated(self._h, n, seed, ctypes.byref(out))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_server_register_generated")
        return int(out.value)

    def register_host(self, values: np.ndarray) -> int:
        values = np.ascontiguousarray(values, dtype=np.float32)
        out = _U64()
        st = _bind_server().rmq_server_register_host(self._h, values.ctypes.data, values.size, ctypes.byref(out))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_server_register_host")
        self._keep[("array", int(out.value))] = values
        return int(out.value)

    def submit(self, array_id: int, lr: np.ndarray, out_idx: np.ndarray | None = None,
               out_min: np.ndarray | None = None) -> int:
        assert lr.dtype == np.uint32 and lr.flags.c_contiguous
        rid = _U64()
        st = _bind_server().rmq_server_submit(
            self._h, array_id, lr.ctypes.data, lr.size // 2,
            out_idx.ctypes.data if out_idx is not None else None,
            out_min.ctypes.data if out_min is not None else None, ctypes.byref(rid))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_server_submit")
        self._keep[("req", int(rid.value))] = (lr, out_idx, out_min)
        return int(rid.value)

    def wait(self, request_id: int, timeout_ms: int = -1) -> tuple[int, float]:
        lat = ctypes.c_double()
        st = _bind_server().rmq_server_wait(self._h, request_id, timeout_ms, ctypes.byref(lat))
        if st != RMQ_ERR_TIMEOUT:
            self._keep.pop(("req", request_id), None)
        return st, float(lat.value)

    def drain(self, timeout_ms: int = -1) -> None:
        st = _bind_server().rmq_server_drain(self._h, timeout_ms)
        if st != RMQ_OK:
            raise RMQError(st, "rmq_server_drain")

    def replay(self, events: np.ndarray, lr: np.ndarray, out_idx: np.ndarray, out_min: np.ndarray):
        assert events.dtype == TRACE_DTYPE
        lat = np.empty(events.size, dtype=np.float64)
        wall = ctypes.c_double()
        st = _bind_server().rmq_server_replay(self._h, events.ctypes.data, events.size, lr.ctypes.data,
                                              out_idx.ctypes.data if out_idx is not None else None,
                                              out_min.ctypes.data if out_min is not None else None,
                                              lat.ctypes.data, ctypes.byref(wall))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_server_replay")
        return lat, float(wall.value)

    def fail_next_batches(self, count: int) -> None:
        """Host-side fault injection: the next `count` batches fail as if
        their upload had returned a CUDA error (their requests get
        RMQ_ERR_CUDA)."""
        st = _bind_server().rmq_server_fail_next_batches(self._h, int(count))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_server_fail_next_batches")

    def stats(self) -> dict:
        s = ServerStats()
        st = _bind_server().rmq_server_get_stats(self._h, ctypes.byref(s))
        if st != RMQ_OK:
            raise RMQError(st, "rmq_server_get_stats")
        return s.as_dict()

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            _bind_server().rmq_server_destroy(self._h)
            self._h = _P()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def serve_serial_loop(handles, events: np.ndarray, lr: np.ndarray, out_idx: np.ndarray,
                      out_min: np.ndarray | None = None) -> float:
    """The server's comparator: the events' query requests one after another
    through rmq_query_idx_host on prebuilt handles (one Hierarchy per array
    id); returns the loop's wall time in seconds."""
    assert events.dtype == TRACE_DTYPE
    arr = (_P * len(handles))(*[h.handle for h in handles])
    wall = ctypes.c_double()
    st = _bind_server().rmq_serve_serial_loop(arr, len(handles), events.ctypes.data, events.size,
                                              lr.ctypes.data if hasattr(lr, "ctypes") else int(lr.data_ptr()),
                                              out_idx.ctypes.data if hasattr(out_idx, "ctypes") else int(out_idx.data_ptr()),
                                              (out_min.ctypes.data if hasattr(out_min, "ctypes") else int(out_min.data_ptr()))
                                              if out_min is not None else None,
                                              ctypes.byref(wall))
    if st != RMQ_OK:
        raise RMQError(st, "rmq_serve_serial_loop")
    return float(wall.value)
