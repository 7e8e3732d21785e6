"""Compile the CUDA library in-tree: simulator_gb300/_lib/libvisgsim.so.

Translation units are compiled in parallel with nvcc for sm_103a only and linked
into one shared library with the CUDA runtime linked statically.  Rebuilds are
skipped when the outputs are newer than every source and header.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libvisgsim.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--threads", "2"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _sources():
    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    cpp = sorted(glob.glob(os.path.join(CSRC, "*.cpp")))
    deps = cu + cpp + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.inl")) + \
        [os.path.join(ROOT, "include", "visg_sim.h")]
    return cu, cpp, deps


def _newer(out: str, deps) -> bool:
    if not os.path.exists(out):
        return False
    t = os.path.getmtime(out)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def build_library(verbose: bool = False, force: bool = False) -> str:
    cu, cpp, deps = _sources()
    os.makedirs(LIBDIR, exist_ok=True)
    if not force and _newer(LIB, deps):
        return LIB
    objs, jobs = [], []
    for src in cu + cpp:
        obj = os.path.join(LIBDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if src.endswith(".cu"):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", src, "-o", obj]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", src, "-o", obj]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
    tmp = LIB + ".tmp"
    _run([nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-Xcompiler", "-fPIC"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_library(verbose=True, force=True))
