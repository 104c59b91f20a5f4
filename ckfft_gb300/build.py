"""Builds ckfft_gb300/libckfft_cuda.so in-tree (sm_103a only).

    python -m ckfft_gb300.build [--force] [-v]

Each .cu / .cpp under csrc/ compiles to an object under _build/ in parallel;
nvcc then links the shared library with the CUDA runtime linked statically,
so the library needs nothing from the Python side at run time.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(HERE, "libckfft_cuda.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libckfft_cuda.so")


def _cuda_include(nvcc: str) -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), "include")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    cpp = sorted(f for f in os.listdir(CSRC) if f.endswith(".cpp"))
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return cu, cpp, headers


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0 or verbose:
        sys.stderr.write(r.stdout + r.stderr)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd[:3])} ... {cmd[-1]}")
    return r.stdout + r.stderr


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compiles stale objects and relinks; returns the library path."""
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    cu, cpp, headers = _sources()
    common = ["-O3", "-std=c++17", f"-I{INCLUDE}", f"-I{CSRC}"]
    jobs = []
    objs = []
    for f in cu:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f[:-3] + ".o")
        objs.append(obj)
        if force or ptxas_info or _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, "-lineinfo", *common, "-Xcompiler", "-fPIC", "-c", src, "-o", obj]
            if ptxas_info:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for f in cpp:
        src = os.path.join(CSRC, f)
        obj = os.path.join(BUILD, f[:-4] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cxx = os.environ.get("CXX", "g++")
            jobs.append([cxx, "-O2", "-std=c++17", "-fPIC", "-Wall", f"-I{_cuda_include(nvcc)}",
                         f"-I{INCLUDE}", f"-I{CSRC}", "-c", src, "-o", obj])
    outputs = []
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
            outputs = list(ex.map(lambda c: _run(c, verbose), jobs))
    if jobs or force or not os.path.exists(LIB):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs], verbose)
    if ptxas_info:
        for o in outputs:
            sys.stdout.write(o)
    build_harness(nvcc, headers, force, verbose)
    return LIB


HARNESS_SRC = os.path.join(HERE, "harness", "ckfft_timing.cpp")
HARNESS = os.path.join(BUILD, "ckfft_timing")


def build_harness(nvcc: str, headers, force: bool = False, verbose: bool = False) -> str:
    """The timing harness executable (_build/ckfft_timing), linked against
    the library in this directory and the CUDA runtime."""
    if not force and not _stale(HARNESS, [HARNESS_SRC, LIB] + headers):
        return HARNESS
    cuda = os.path.dirname(_cuda_include(nvcc))
    lib64 = os.path.join(cuda, "lib64")
    cxx = os.environ.get("CXX", "g++")
    _run([cxx, "-O2", "-std=c++17", "-Wall", f"-I{INCLUDE}", f"-I{_cuda_include(nvcc)}", HARNESS_SRC,
          "-o", HARNESS, f"-L{HERE}", "-l:libckfft_cuda.so", f"-L{lib64}", "-lcudart",
          "-Wl,-rpath,$ORIGIN/..", f"-Wl,-rpath,{lib64}"], verbose)
    return HARNESS


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true", help="print registers/spills per kernel")
    a = ap.parse_args()
    print(build(force=a.force, verbose=a.verbose, ptxas_info=a.ptxas_info))


if __name__ == "__main__":
    main()
