"""Host code under AddressSanitizer and UBSan, CPU only (skipped where the compiler has
no sanitizer runtime):

* the mesh code (OBJ reader, mesh transforms, spring and seam builders), driven by
  tests/fuzz_mesh.cpp: the reference's own OBJ files when they are on this machine,
  mutated OBJ files, and random triangle soups;
* the oracle, driven by tests/oracle_sanitize.cpp through its C interface."""
import glob
import os
import shutil
import subprocess

import pytest

from oracle.build import REFERENCE

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_mesh_code_under_sanitizers(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    exe = tmp_path / "fuzz_mesh"
    src = [os.path.join(HERE, "fuzz_mesh.cpp"), os.path.join(ROOT, "simulator_gb300", "csrc", "visg_mesh.cpp"),
           os.path.join(ROOT, "simulator_gb300", "csrc", "visg_host.cpp")]
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           "-I", os.path.join(ROOT, "include"), *src, "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if "asan" in r.stderr.lower() or "ubsan" in r.stderr.lower() or "sanitize" in r.stderr.lower():
            pytest.skip("no sanitizer runtime: " + r.stderr.strip().splitlines()[-1])
        raise AssertionError(r.stderr)
    meshes = sorted(glob.glob(os.path.join(REFERENCE, "resources", "**", "*.obj"), recursive=True))
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1")
    r = subprocess.run([str(exe), str(tmp_path / "fuzz.obj"), *meshes], capture_output=True, text=True, env=env,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "fuzz_mesh: clean" in r.stdout


def test_oracle_under_sanitizers(tmp_path):
    """The oracle itself (the checker) under AddressSanitizer and UBSan, driven by
    tests/oracle_sanitize.cpp through its C interface."""
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    exe = tmp_path / "oracle_sanitize"
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           "-fopenmp", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
           os.path.join(HERE, "oracle_sanitize.cpp"), os.path.join(ROOT, "oracle", "visg_oracle.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        if "asan" in r.stderr.lower() or "ubsan" in r.stderr.lower() or "sanitize" in r.stderr.lower():
            pytest.skip("no sanitizer runtime: " + r.stderr.strip().splitlines()[-1])
        raise AssertionError(r.stderr)
    env = dict(os.environ, OMP_NUM_THREADS="2", ASAN_OPTIONS="detect_leaks=1:abort_on_error=1")
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "oracle_sanitize: clean" in r.stdout
