"""Build libnatural_gb300.so in-tree for sm_103a.

nvcc compiles the CUDA translation units with `-gencode
arch=compute_103a,code=sm_103a`; g++ compiles the host C++; nvcc links the
shared library against the static CUDA runtime.  Units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libnatural_gb300.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = shutil.which("nvcc") or os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["ntt.cu", "carry.cu", "batch.cu", "noalloc.cu", "decimal.cu"]
CPP_SOURCES = ["engine.cpp", "profile.cpp", "natural_ops.cpp", "serve.cpp", "series.cpp", "host_glue.cpp", "divide.cpp",
               "host_pool.cpp"]
HEADERS = ["nn_device.cuh", "nn_internal.h", "ntt_tiles.cuh", "scan_tiles.cuh", "tma.cuh", "context_access.h",
           "../../include/natural_gb300.hpp"]


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _compile(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "natural_gb300.h")]
    jobs, objs = [], []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++20", "-Xcompiler", "-fPIC",
                         "--expt-relaxed-constexpr", "-rdc=false", "-c", s, "-o", o])
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append(["g++", "-O2", "-std=c++20", "-fPIC", "-Wall", "-I", os.path.join(CUDA_HOME, "include"),
                         "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
            for f in [ex.submit(_compile, j) for j in jobs]:
                f.result()
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        _compile([NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-cudart", "static"])
        os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
