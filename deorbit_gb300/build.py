"""Build libdeorbit_sph.so (sm_103a) in-tree: deorbit_gb300/_lib/libdeorbit_sph.so.

Translation units compile in parallel with nvcc; no cmake, one -gencode.
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
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libdeorbit_sph.so")

SOURCES = ["scan_sort.cu", "engine_fp64.cu", "engine_mixed.cu", "capi.cu", "cell_sort_api.cu", "serve.cpp",
           "euler.cu", "euler_mixed.cu"]
# Per-source flags: the grid solver evaluates every expression in the
# reference's operation order, without fused multiply-adds.
SOURCE_FLAGS = {"euler.cu": ["--fmad=false"]}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: host code (flaw seeding, file formats) gives the same
# results on x86 and on Arm, where g++ would otherwise fuse a*b+c.
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".hpp"))] + [
        os.path.join(ROOT, "include", "deorbit_sph.h"), os.path.join(ROOT, "include", "deorbit_euler.h")]


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nv = nvcc()
    hdrs = _headers()
    objs = []
    jobs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or not _newer(o, [s] + hdrs):
            jobs.append([nv] + NVCC_FLAGS + SOURCE_FLAGS.get(src, []) + ARCH + ["-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f"nvcc failed for {cmd[-3]}")
    if force or jobs or not _newer(LIB, objs):
        cmd = [nv, "-shared"] + ARCH + ["-o", LIB] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode != 0:
            raise RuntimeError("link failed")
    build_cli(verbose, force)
    return LIB


CLI = os.path.join(LIBDIR, "gpu_ic")


def build_cli(verbose: bool = False, force: bool = False) -> str:
    """The gpu_ic command-line driver (host C++ over the C ABI)."""
    src = os.path.join(CSRC, "gpu_ic.cpp")
    if not force and _newer(CLI, [src, LIB, os.path.join(ROOT, "include", "deorbit_sph.h")]):
        return CLI
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-I", os.path.join(ROOT, "include"), src,
           "-o", CLI, "-L", LIBDIR, "-ldeorbit_sph", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose or r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError("gpu_ic build failed")
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
