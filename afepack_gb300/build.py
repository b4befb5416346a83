"""Builds libafepack_gb300.so in-tree with nvcc for sm_103a.

    python -m afepack_gb300.build [--force]

Each translation unit is compiled in parallel; the element-matrix / scatter
and Galerkin-product units are compiled with -fmad=false because their
floating-point operations must round exactly like AFEPack's host code.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libafepack_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = [
    # (file, extra flags)
    ("context.cu", []),
    ("assemble.cu", ["-fmad=false"]),
    ("rap.cu", ["-fmad=false"]),
    ("coarsen.cu", ["-fmad=false"]),
    ("solve.cu", []),
    ("amg.cu", []),
    ("mrhs.cu", []),
    ("vcycle_stream.cu", []),
    ("noalloc.cu", []),
    ("coarsen_host.cpp", []),
    ("server.cpp", []),
]
HEADERS = ["common.cuh", "kernels.cuh", "solve.cuh", "amg_internal.cuh", "launch.cuh", "quadrature_tables.h"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "afepack_gb300.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src: str, flags: list[str], obj: str) -> None:
    path = os.path.join(CSRC, src)
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
               *flags, "-c", path, "-o", obj]
    else:
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-fPIC", "-I" + os.path.join(_cuda_home(), "include"), *flags, "-c", path,
               "-o", obj]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    objs, jobs = [], []
    for src, flags in SOURCES:
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, os.path.join(CSRC, src)):
            jobs.append((src, flags, obj))
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            futs = [ex.submit(_compile, *j) for j in jobs]
            for f in futs:
                f.result()
    if force or jobs or not os.path.exists(LIB):
        cmd = [_nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
