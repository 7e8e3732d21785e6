"""The oracle against golden fixtures produced by the reference's own kernels.

The reference has no tests or golden vectors, so its hot-path kernels (verlet,
compute_morton_bbox, processInternalNode, calculateBoudingBox, D_BVH::intersect,
Primitive::d_intersect), compiled unmodified for sm_103a, were run on a GB300 by
tests/golden/make_golden.py and their outputs committed here.  The CPU oracle must
reproduce them bit for bit: the LBVH of three bodies and a 200-step trajectory
with contacts.  This pins the oracle that the GPU tests compare the library with.
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

from oracle.ffi import OracleSim
from simulator_gb300 import scenes
from simulator_gb300.params import VisgParams, reference_params

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
LBVH = sorted(glob.glob(os.path.join(GOLDEN, "lbvh_*.npz")))
TRAJ = sorted(glob.glob(os.path.join(GOLDEN, "traj_*.npz")))


def test_fixtures_present():
    assert len(LBVH) >= 3 and len(TRAJ) >= 1


@pytest.mark.parametrize("path", LBVH, ids=[os.path.basename(p) for p in LBVH])
def test_oracle_lbvh_matches_reference_kernels(path):
    g = np.load(path)
    cloth = scenes.grid_cloth(4, 1.0, 5.0, pin_top_corners=False)
    p = reference_params(3)
    p.box_depth = float(g["box_depth"])
    o = OracleSim(p, cloth.xyz, cloth.lists, g["body_xyz"], g["body_tris"], None, prec=4)
    b = o.export_lbvh()
    assert b["n_leaves"] == int(g["n_leaves"])
    for k in ("tri_codes", "sorted_codes", "sorted_tris", "child_a", "child_b", "parent_internal", "parent_leaf"):
        assert np.array_equal(b[k], g[k]), k
    for k in ("tri_boxes", "leaf_boxes", "internal_boxes", "root_box"):
        assert np.array_equal(b[k], g[k]), k


@pytest.mark.parametrize("path", TRAJ, ids=[os.path.basename(p) for p in TRAJ])
def test_oracle_trajectory_matches_reference_kernels(path):
    g = np.load(path)
    raw = g["params"].tobytes()  # the struct as written; fields added later are appended (zero)
    raw = raw + bytes(max(0, C.sizeof(VisgParams) - len(raw)))
    p = VisgParams.from_buffer_copy(raw[: C.sizeof(VisgParams)])
    lists = []
    for l in (0, 1):
        ent = np.zeros(len(g[f"end{l}"]), scenes.SPRING_DTYPE)
        ent["end"], ent["rest"] = g[f"end{l}"], g[f"rest{l}"]
        lists.append(scenes.SpringList(g[f"row{l}"], ent))
    o = OracleSim(p, g["cloth_xyz"], lists, g["body_xyz"], g["body_tris"], g["body_normals"], prec=4)
    done = 0
    for k in (1, 50, 100, 200):
        o.step(k - done)
        done = k
        x, xo, n = (a.astype(np.float32) for a in o.state())
        assert np.array_equal(x, g[f"x_{k}"]), k
        assert np.array_equal(xo, g[f"xo_{k}"]), k
        assert np.array_equal(n, g[f"n_{k}"]), k
    assert (np.abs(g["n_200"]).sum(1) > 0).sum() > 0, "the fixture must include contacts"
