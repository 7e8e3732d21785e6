"""Build recipe of the checkers (test infrastructure only).

  oracle/_build/libvisg_oracle.so   the CPU restatement (visg_oracle.cpp), g++ -fopenmp,
                                    -ffp-contract=off so float arithmetic is one IEEE
                                    operation per source operation on x86 and Arm alike
  oracle/_build/librefharness.so    host loader of the reference's kernels (refkern/refharness.cpp)
  oracle/_ref/refkern.cubin         the reference's own hot-path kernels (verlet.cu,
                                    bvh/cudaBRT.cu, bvh/primitive.cu and bvh/bvh.cu) compiled
                                    for sm_103a with --fmad=false from the reference tree.  Built
                                    only where the reference tree exists; the cubin is device
                                    code and travels to the GPU machine with the repository.

bvh.cu does not compile as shipped (bvh.cu:33 declares `float x = p.x, float y = ...`);
the recipe writes a corrected copy of that one file into oracle/_ref/gen/, compiles, and
deletes the copy.  Nothing from the reference tree is kept in the repository.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
CUBIN = os.path.join(REF_OUT, "refkern.cubin")
ORACLE_SO = os.path.join(BUILD, "libvisg_oracle.so")
HARNESS_SO = os.path.join(BUILD, "librefharness.so")
# the reference tree: VISG_REFERENCE_DIR, else a checkout named "reference" beside
# the repository
REFERENCE = os.environ.get("VISG_REFERENCE_DIR",
                           os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=cwd)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(force=False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "visg_oracle.cpp")
    hdr = os.path.join(os.path.dirname(HERE), "include", "visg_sim.h")
    if force or _stale(ORACLE_SO, [src, hdr]):
        _run(["g++", "-O2", "-ffp-contract=off", "-fopenmp", "-std=c++17", "-shared", "-fPIC", "-o",
              ORACLE_SO + ".tmp", src])
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def build_harness(force=False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "refkern", "refharness.cpp")
    if force or _stale(HARNESS_SO, [src]):
        lib64 = os.path.join(CUDA, "lib64")
        stubs = os.path.join(lib64, "stubs")
        _run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-shared", "-fPIC", f"-I{CUDA}/include", "-o",
              HARNESS_SO + ".tmp", src, f"-L{lib64}", f"-L{stubs}", "-lcudart_static", "-lcuda", "-ldl", "-lrt",
              "-lpthread"])
        os.replace(HARNESS_SO + ".tmp", HARNESS_SO)
    return HARNESS_SO


def build_refkern(force=False) -> str | None:
    """Compile the reference's kernels into oracle/_ref/refkern.cubin (needs the tree)."""
    src_dir = os.path.join(REFERENCE, "src")
    if not os.path.isdir(src_dir):
        return CUBIN if os.path.exists(CUBIN) else None
    unity = os.path.join(HERE, "refkern", "refkern_unity.cu")
    deps = [unity, os.path.join(HERE, "refkern", "include", "glm", "glm.hpp")]
    if not force and not _stale(CUBIN, deps):
        return CUBIN
    gen = os.path.join(REF_OUT, "gen")
    os.makedirs(gen, exist_ok=True)
    with open(os.path.join(src_dir, "bvh", "bvh.cu"), "r", encoding="latin-1") as f:
        text = f.read()
    bad = "float x = p.x, float y = p.y, float z = p.z;"
    if bad not in text:
        raise RuntimeError("bvh.cu: expected declaration at line 33 not found")
    with open(os.path.join(gen, "bvh_fixed.cu"), "w", encoding="latin-1") as f:
        f.write(text.replace(bad, "float x = p.x, y = p.y, z = p.z;"))
    try:
        _run([os.path.join(CUDA, "bin", "nvcc"), "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
              "--fmad=false", "-O3", "-std=c++17", "-w", "-I", os.path.join(HERE, "refkern", "include"), "-I", gen,
              "-I", os.path.join(src_dir, "bvh"), "-I", src_dir, "-o", CUBIN + ".tmp", unity])
        os.replace(CUBIN + ".tmp", CUBIN)
    finally:
        shutil.rmtree(gen, ignore_errors=True)
    return CUBIN


def build_all(force=False):
    out = {"oracle": build_oracle(force), "harness": build_harness(force), "refkern": build_refkern(force)}
    return out


if __name__ == "__main__":
    print(build_all(force=True))
