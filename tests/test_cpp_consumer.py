"""A compiled C++ consumer of the C ABI (tests/consumer/scene_consumer.cpp).

The program includes only include/visg_sim.h and links -lvisgsim, and drives the
library as the reference's Scene drives its Simulator (scene.cpp:176-186, 267-276,
357, 85): OBJ meshes, the reference's spring lists, create, a step and the output
stage per frame, one dragged vertex, destroy.

CPU: the program compiles and links against the header and the built library, and,
with no GPU, fails loudly (status VISG_ERR_NO_DEVICE from visg_create, exit 2)
instead of computing anything on the host.
GPU: its final positions and last frame's output stage equal, bit for bit, the same
sequence run through the Python (ctypes) binding.
"""
import os
import subprocess

import numpy as np
import pytest

import simulator_gb300 as vs
from simulator_gb300 import scenes
from simulator_gb300._build import LIBDIR

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "consumer", "scene_consumer.cpp")

FRAMES, DRAG_FRAME, DRAG_VERTEX, DY = 150, 60, 17, 0.02


def build_consumer(tmp_path) -> str:
    vs.lib()  # the library is built
    exe = str(tmp_path / "scene_consumer")
    cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), SRC, "-o", exe, "-L", LIBDIR,
           "-lvisgsim", f"-Wl,-rpath,{LIBDIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def write_meshes(tmp_path):
    cloth = scenes.grid_cloth(24, 1.0, 0.0, pin_top_corners=False)
    body = scenes.icosphere(3, 0.3, (0.0, -0.31, 0.0))
    vs.write_obj(str(tmp_path / "cloth.obj"), cloth.xyz, cloth.faces)
    with open(tmp_path / "body.obj", "w") as f:  # with per-vertex normals, "a/t/n" faces
        for p in body.xyz:
            f.write(f"v {p[0]:.9g} {p[1]:.9g} {p[2]:.9g}\n")
        for nv in body.normals:
            f.write(f"vn {nv[0]:.9g} {nv[1]:.9g} {nv[2]:.9g}\n")
        for t in body.tris.astype(np.int64) + 1:
            f.write(f"f {t[0]}/1/{t[0]} {t[1]}/1/{t[1]} {t[2]}/1/{t[2]}\n")
    return str(tmp_path / "cloth.obj"), str(tmp_path / "body.obj")


def run_consumer(exe, cloth_obj, body_obj, out):
    return subprocess.run([exe, cloth_obj, body_obj, str(FRAMES), str(DRAG_FRAME), str(DRAG_VERTEX), str(DY), out],
                          capture_output=True, text=True, timeout=300)


def test_consumer_compiles_links_and_fails_loudly_without_a_gpu(tmp_path):
    from conftest import has_gpu
    exe = build_consumer(tmp_path)
    if has_gpu():
        pytest.skip("a GPU is visible: the GPU test runs the consumer")
    cloth_obj, body_obj = write_meshes(tmp_path)
    r = run_consumer(exe, cloth_obj, body_obj, str(tmp_path / "out.bin"))
    assert r.returncode == 2, (r.returncode, r.stdout, r.stderr)
    assert "visg_create failed (-4)" in r.stderr  # VISG_ERR_NO_DEVICE: no host fallback
    assert not os.path.exists(tmp_path / "out.bin")


@pytest.mark.gpu
def test_consumer_equals_python_binding(tmp_path):
    exe = build_consumer(tmp_path)
    cloth_obj, body_obj = write_meshes(tmp_path)
    out = str(tmp_path / "out.bin")
    r = run_consumer(exe, cloth_obj, body_obj, out)
    assert r.returncode == 0, r.stderr
    print(r.stdout.strip())
    raw = np.fromfile(out, np.uint8)
    n = int(raw[:4].view(np.int32)[0])
    body = raw[4:].view(np.float32)
    x, pos4, vn = body[:3 * n].reshape(n, 3), body[3 * n:7 * n].reshape(n, 4), body[7 * n:].reshape(n, 3)

    cx, _, cf = vs.load_obj(cloth_obj)
    bx, bn, bf = vs.load_obj(body_obj)
    p = vs.reference_params(2)
    sim = vs.Simulator(cx, vs.springs_from_mesh(cx, cf), bx, bf, bn, params=p)
    sim.set_faces(cf)
    for f in range(FRAMES):
        if f == DRAG_FRAME:
            t = sim.positions()[DRAG_VERTEX].copy()
            t[1] = np.float32(t[1] + np.float32(DY))
            sim.update_vertex(t, DRAG_VERTEX)
        sim.simulate(1)
        ref_pos4, ref_vn, _ = sim.render()
    ref_x = sim.positions()
    assert sim.count_contacts() > 0
    sim.close()
    assert np.array_equal(x, ref_x)
    assert np.array_equal(pos4, ref_pos4)
    assert np.array_equal(vn, ref_vn, equal_nan=True)
