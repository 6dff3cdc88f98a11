"""The reference's own GPU kernels, run through the CUDA driver API
(TEST / BENCHMARK INFRASTRUCTURE ONLY).

oracle/build_ref.sh compiles the reference's hierarchical kernels from its
sources (src/xxx.h, paper configurations; see ref_gpu_harness.cu) into a
device-only fatbin, oracle/_ref/rmq_ref_kernels.fatbin.  Device code does not
depend on the host architecture, so the same file runs wherever a GB300 is.
This module loads it (cuModuleLoad, kernel handles by name through
cuModuleEnumerateFunctions / cuFuncGetName) and reproduces the launches of the
reference's host drivers:

  CL, alg 16  xxx_rmq (src/xxx.h:203-298): layout loop :225-243, one
              xxx_build_step<.., 4, 1> launch per level with
              grid = ceil(min(size_{k+1} << 4, 2^30) / 1024) x 1024 (:258-265),
              then xxx_query<.., 4, 1> with grid ceil(q / 1024) x 1024 (:276-281)
  VL, alg 20  hierarchical_vector_load (src/xxx.h:932-1040): same layout with
              rf 8, xxx_build_step<.., 2, 1> per level (:996-1003), then
              kernel_hierarchical_vector_load<.., 1> (:1015-1019)

Used only to check parity against, and to time, the reference's GPU path on
the same GPU as this library's kernels.  Arrays must hold a multiple of 4
values (the reference's VL kernel reads whole float4s past n otherwise).
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import oracle

FATBIN = Path(__file__).resolve().parent / "_ref" / "rmq_ref_kernels.fatbin"
BSIZE = 1024  # the reference's block size (CMakeLists.txt:53-55)


class _Metadata(ctypes.Structure):
    """xxx_metadata_type<uint32_t, uint2> (src/constants.cuh:34-39)."""
    _fields_ = [("num_levels", ctypes.c_uint32), ("level_offset", ctypes.c_uint32 * 20),
                ("level_size", ctypes.c_uint32 * 20)]


def available() -> bool:
    return FATBIN.exists()


class RefKernels:
    def __init__(self):
        import torch
        if not FATBIN.exists():
            raise RuntimeError(f"{FATBIN} missing (reference sources were not available to build it)")
        torch.cuda.init()
        torch.empty(1, device="cuda")  # primary context current on this thread
        cu = ctypes.CDLL("libcuda.so.1")
        self.cu = cu
        mod = ctypes.c_void_p()
        self._check(cu.cuModuleLoad(ctypes.byref(mod), str(FATBIN).encode()), "cuModuleLoad")
        self.mod = mod
        count = ctypes.c_uint()
        self._check(cu.cuModuleGetFunctionCount(ctypes.byref(count), mod), "cuModuleGetFunctionCount")
        funcs = (ctypes.c_void_p * count.value)()
        self._check(cu.cuModuleEnumerateFunctions(funcs, count, mod), "cuModuleEnumerateFunctions")
        names = {}
        for f in funcs:
            nm = ctypes.c_char_p()
            self._check(cu.cuFuncGetName(ctypes.byref(nm), ctypes.c_void_p(f)), "cuFuncGetName")
            names[nm.value.decode()] = ctypes.c_void_p(f)
        self.names = names

        def pick(*parts):
            hits = [v for k, v in names.items() if all(p in k for p in parts)]
            if len(hits) != 1:
                raise RuntimeError(f"kernel {parts} not found uniquely in {sorted(names)}")
            return hits[0]

        self.cl_build = pick("xxx_build_step", "Lj4ELj1E")
        self.cl_query = pick("xxx_query", "Lj4ELj1E")
        self.vl_build = pick("xxx_build_step", "Lj2ELj1E")
        self.vl_query = pick("kernel_hierarchical_vector_load")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed: CUresult {rc}")

    def _launch(self, f, grid, args, stream):
        params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p) for a in args])
        self._check(self.cu.cuLaunchKernel(f, ctypes.c_uint(grid), ctypes.c_uint(1), ctypes.c_uint(1),
                                           ctypes.c_uint(BSIZE), ctypes.c_uint(1), ctypes.c_uint(1),
                                           ctypes.c_uint(0), ctypes.c_void_p(stream), params, None),
                    "cuLaunchKernel")

    def build(self, values, t: int, variant: str, stream: int):
        """Builds the reference's level buffer for `values` (CUDA float32
        tensor); returns (metadata, level buffer tensor)."""
        import torch
        n = values.numel()
        if n % 4:
            raise ValueError("the reference's VL kernel needs n % 4 == 0")
        cg_log, rf_log = (4, 5) if variant == "cl" else (2, 3)
        k, sizes, offs = oracle.layout(n, t, rf_log)
        md = _Metadata()
        md.num_levels = k
        for i in range(k):
            md.level_size[i] = sizes[i]
            md.level_offset[i] = 0xFFFFFFFF if i == 0 else offs[i]
        total = offs[-1] + sizes[-1] if k > 1 else 0
        lvl = torch.empty(total + 64, dtype=torch.float32, device=values.device)  # +64: float4 tail reads
        f = self.cl_build if variant == "cl" else self.vl_build
        for lev in range(k - 1):
            src = values.data_ptr() if lev == 0 else lvl.data_ptr() + 4 * offs[lev]
            dst = lvl.data_ptr() + 4 * offs[lev + 1]
            threads = min(sizes[lev + 1] << cg_log, (0x7FFFFFFF >> 1) + 1)
            self._launch(f, (threads + BSIZE - 1) // BSIZE,
                         [ctypes.c_void_p(src), ctypes.c_void_p(dst), ctypes.c_uint32(sizes[lev]),
                          ctypes.c_uint32(sizes[lev + 1])], stream)
        return md, lvl

    def query(self, values, md, lvl, lr, out, t: int, variant: str, stream: int):
        """One query launch of the reference's CL or VL kernel (minima into out)."""
        q = lr.numel() // 2
        grid = (q + BSIZE - 1) // BSIZE
        if variant == "cl":
            args = [ctypes.c_uint32(q), ctypes.c_void_p(lr.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                    ctypes.c_void_p(values.data_ptr()), ctypes.c_void_p(lvl.data_ptr()), md, ctypes.c_uint32(t)]
            self._launch(self.cl_query, grid, args, stream)
        else:
            args = [ctypes.c_uint32(values.numel() >> 2), ctypes.c_uint32(q), ctypes.c_void_p(lr.data_ptr()),
                    ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(values.data_ptr()),
                    ctypes.c_void_p(lvl.data_ptr()), md, ctypes.c_uint32(t)]
            self._launch(self.vl_query, grid, args, stream)


def time_reference(values, lr, variant: str, t: int, steps: int = 5, warmup: int = 3):
    """Times the reference's query kernel (CUDA events, warm); returns
    (queries/s, minima tensor)."""
    import torch
    rk = RefKernels()
    stream = torch.cuda.current_stream().cuda_stream
    md, lvl = rk.build(values, t, variant, stream)
    out = torch.empty(lr.numel() // 2, dtype=torch.float32, device=values.device)
    for _ in range(warmup):
        rk.query(values, md, lvl, lr, out, t, variant, stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        rk.query(values, md, lvl, lr, out, t, variant, stream)
    e1.record()
    torch.cuda.synchronize()
    return (lr.numel() // 2) * steps / (e0.elapsed_time(e1) / 1e3), out
