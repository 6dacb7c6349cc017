"""Build libsjbg.so (the C-ABI stream-join library) for sm_103a, in-tree.

    python gpu-stream-join-benchmark_gb300/build.py [--force]

Every csrc/*.cu translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`` and linked into
``lib/libsjbg.so``; the C++ host harness (host/) is built into
``lib/runExperiment``.  Objects go to ``_build/`` (git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libsjbg.so")
HARNESS = os.path.join(LIBDIR, "runExperiment")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
                     "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers() -> list[str]:
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(ROOT, "include", "*.h")))


def _compile(src: str, force: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src).replace(".cu", ".o"))
    if not force and _newer(obj, [src] + _headers()):
        return obj
    cmd = [nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_lib(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force), srcs))
    if force or not _newer(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def build_harness(force: bool = False) -> str | None:
    """The C++ runExperiment harness over the C ABI (host/*.cpp)."""
    srcs = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    if not srcs:
        return None
    deps = srcs + glob.glob(os.path.join(HOST, "*.hpp")) + [LIB]
    if not force and _newer(HARNESS, deps):
        return HARNESS
    cxx = shutil.which("g++") or "g++"
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc())))
    cudalib = os.path.join(cuda, "lib64")
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", HOST,
           "-I", os.path.join(cuda, "include")] + srcs + [
        "-o", HARNESS, "-L", LIBDIR, "-lsjbg", "-Wl,-rpath,$ORIGIN", "-L", cudalib, "-lcudart",
        "-Wl,-rpath," + cudalib, "-lpthread", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"harness build failed:\n{r.stdout}\n{r.stderr}")
    return HARNESS


def build(force: bool = False) -> str:
    lib = build_lib(force)
    build_harness(force)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
