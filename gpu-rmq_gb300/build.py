"""Build recipe for the GB300 RMQ library, its driver and the test oracle.

Everything is compiled in-tree with nvcc / g++ / gcc (no cmake), translation
units in parallel, one -gencode (sm_103a).  Outputs:

  gpu-rmq_gb300/librmq_gb300.so      CUDA kernels + C ABI (include/rmq_gb300.h)
  gpu-rmq_gb300/librmq_gb300_checked.so  the same with bounds-checked level loads
                                     (RMQ_DEBUG_BOUNDS=1; tests only)
  gpu-rmq_gb300/librmq_gen.so        host input generators (include/rmq_gb300_gen.h)
  gpu-rmq_gb300/driver/rtxrmq        the benchmark driver (reference CLI)
  oracle/liboracle.so                CPU oracle (test infrastructure)
  oracle/_ref/librmq_ref.so          reference build for pinning (only when
                                     RMQ_REFERENCE_ROOT names the reference checkout)
"""
from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
DRIVER = PKG / "driver"
INCLUDE = ROOT / "include"
ORACLE = ROOT / "oracle"
BUILD = PKG / "_build" / platform.machine()

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CUDA_SOURCES = ["rmq_build.cu", "rmq_query.cu", "rmq_api.cu", "rmq_noalloc.cu", "rmq_batch.cu",
                "rmq_gen_device.cu", "rmq_serve.cu", "rmq_probe.cu"]

LIB = PKG / "librmq_gb300.so"
CHECKED_LIB = PKG / "librmq_gb300_checked.so"  # bounds-checked build (tests only)
GENLIB = PKG / "librmq_gen.so"
DRIVER_BIN = DRIVER / "rtxrmq"
ORACLE_LIB = ORACLE / "liboracle.so"
REF_LIB = ORACLE / "_ref" / "librmq_ref.so"


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the RMQ library")
    return cand


_ELF_MACHINE = {"x86_64": 62, "aarch64": 183, "arm64": 183}


def _foreign_binary(path: Path) -> bool:
    """True for an ELF file built for another CPU architecture (a tree copied
    between an x86 build host and an Arm GPU host keeps stale binaries)."""
    want = _ELF_MACHINE.get(platform.machine())
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return False
    if want is None or len(head) < 20 or head[:4] != b"\x7fELF":
        return False
    return int.from_bytes(head[18:20], "little") != want


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists() or _foreign_binary(out):
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def build_library(force: bool = False) -> Path:
    """The library and, from the same sources with RMQ_DEBUG_BOUNDS=1, its
    bounds-checked twin (all translation units compiled in parallel)."""
    nvcc = _nvcc()
    hdrs = _headers()
    jobs = []
    variants = [(LIB, BUILD, []), (CHECKED_LIB, BUILD / "checked", ["-DRMQ_DEBUG_BOUNDS=1"])]
    links = []
    for lib, outdir, flags in variants:
        outdir.mkdir(parents=True, exist_ok=True)
        objs = []
        for src in CUDA_SOURCES:
            s = CSRC / src
            o = outdir / (s.stem + ".o")
            objs.append(o)
            if force or _stale(o, [s] + hdrs):
                jobs.append([nvcc, *ARCH, *NVCC_FLAGS, *flags, "-c", str(s), "-o", str(o)])
        links.append((lib, objs))
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for f in [ex.submit(_run, j) for j in jobs]:
            f.result()
    for lib, objs in links:
        if force or _stale(lib, objs):
            _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs)])
    return LIB


def build_generators(force: bool = False) -> Path:
    src = DRIVER / "rmq_gen.cpp"
    if force or _stale(GENLIB, [src, INCLUDE / "rmq_gb300_gen.h"]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", str(src), "-o", str(GENLIB)])
    return GENLIB


def build_driver(force: bool = False) -> Path:
    srcs = [DRIVER / "rtxrmq.cpp", DRIVER / "rmq_gen.cpp"]
    if not srcs[0].exists():
        return DRIVER_BIN
    deps = srcs + _headers() + [LIB]
    if force or _stale(DRIVER_BIN, deps):
        _run([_nvcc(), "-O2", "-std=c++17", "-Xcompiler", "-fopenmp", *map(str, srcs),
              "-o", str(DRIVER_BIN), "-L" + str(PKG), "-lrmq_gb300", "-lgomp",
              "-Xlinker", "-rpath=$ORIGIN/..", "-Xlinker", "-rpath=" + str(PKG)])
    return DRIVER_BIN


def build_oracle(force: bool = False) -> Path:
    """The oracle (C scan and sparse table, C++ generators) as one library."""
    src_c, src_cpp = ORACLE / "rmq_oracle.c", ORACLE / "rmq_oracle_gen.cpp"
    if force or _stale(ORACLE_LIB, [src_c, src_cpp]):
        BUILD.mkdir(parents=True, exist_ok=True)
        obj_c, obj_cpp = BUILD / "rmq_oracle.o", BUILD / "rmq_oracle_gen.o"
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-fopenmp", "-c", str(src_c), "-o", str(obj_c)])
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-c", str(src_cpp), "-o", str(obj_cpp)])
        _run(["g++", "-shared", "-fopenmp", str(obj_c), str(obj_cpp), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def build_reference(force: bool = False, reference_root: str | None = None) -> Path | None:
    """Compiles the reference's own CPU path for pinning, when a reference
    checkout is named (the argument, else the environment variable
    RMQ_REFERENCE_ROOT)."""
    root = reference_root or os.environ.get("RMQ_REFERENCE_ROOT")
    if not root:
        return None
    ref = Path(root)
    if not (ref / "src" / "cpu_methods.h").exists():
        return None
    deps = [ORACLE / "ref_harness.cu", ORACLE / "ref_gpu_harness.cu", ORACLE / "build_ref.sh"]
    if force or _stale(REF_LIB, deps):
        _run(["bash", str(ORACLE / "build_ref.sh"), str(ref)])
    return REF_LIB


def build_all(force: bool = False, reference_root: str | None = None) -> None:
    with ThreadPoolExecutor(max_workers=4) as ex:
        futs = [ex.submit(build_library, force), ex.submit(build_generators, force),
                ex.submit(build_oracle, force), ex.submit(build_reference, force, reference_root)]
        for f in futs:
            f.result()
    build_driver(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built:", LIB, GENLIB, DRIVER_BIN, ORACLE_LIB)
