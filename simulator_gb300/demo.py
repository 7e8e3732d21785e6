"""Headless run of a garment OBJ over a body OBJ: the reference's demo
(src/main.cpp:24-32, src/scene.cpp) without the window.

    python -m simulator_gb300.demo --cloth tshirt2.obj --body female.obj \\
        --reference-pose --steps 2000 --out frames/

Reads both meshes (visg_obj_load), applies the demo's placement with
--reference-pose (the garment rotated 90 degrees about x and -4 about z, scaled by
3.33 and raised by (0, 1.98, 0.02); the body scaled by 3.226 and raised by
(0, 1.8, 0)), builds the reference's two spring lists from the garment's triangles,
(sewing the pieces of a multi-piece garment, as the reference does for
SINGLE_LAYER_BOUNDARY meshes) and steps the simulator with the reference's constants, writing the garment as
an OBJ every --every steps (positions and triangles) and printing the throughput.
"""
from __future__ import annotations

import argparse
import os
import time

import numpy as np

import simulator_gb300 as vs


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--cloth", required=True)
    ap.add_argument("--body", required=True)
    ap.add_argument("--reference-pose", action="store_true")
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--every", type=int, default=0, help="write the garment every N steps (0: at the end)")
    ap.add_argument("--out", default="demo_out")
    a = ap.parse_args(argv)
    cloth, _, cf = vs.load_obj(a.cloth)
    body, bn, bf = vs.load_obj(a.body)
    if a.reference_pose:
        vs.mesh_rotate(cloth, 90, 0)
        vs.mesh_rotate(cloth, -4, 2)
        vs.mesh_scale(cloth, 3.33)
        vs.mesh_translate(cloth, 0, 1.98, 0.02)
        vs.mesh_scale(body, 3.226)
        vs.mesh_translate(body, 0, 1.8, 0)
    groups = vs.obj_groups(a.cloth)  # a multi-piece garment ("# object" groups) is sewn
    lists = vs.springs_from_mesh_sewn(cloth, cf, groups) if len(groups) >= 2 else vs.springs_from_mesh(cloth, cf)
    sim = vs.Simulator(cloth, lists, body, bf, bn, params=vs.reference_params(2))
    sim.set_faces(cf)
    os.makedirs(a.out, exist_ok=True)
    every = a.every if a.every > 0 else a.steps
    done, t0 = 0, time.perf_counter()
    while done < a.steps:
        k = min(every, a.steps - done)
        sim.simulate(k)
        done += k
        x = sim.positions()
        vs.write_obj(os.path.join(a.out, f"cloth_{done:06d}.obj"), x, cf)
    el = time.perf_counter() - t0
    print(f"{len(cloth)} garment vertices, {len(bf)} body triangles, {a.steps} steps in {el:.2f} s "
          f"({len(cloth) * a.steps / el:.3g} vertex-steps/s incl. writing), contacts {sim.count_contacts()}")
    sim.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
