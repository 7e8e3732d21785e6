"""Generate the golden fixtures of tests/golden/ with the reference's own kernels.

Runs where the reference-kernel cubin was built and a GPU is present:

    python tests/golden/make_golden.py OUT_DIR

Every fixture holds its inputs and the reference kernels' outputs (refkern: the
reference's verlet / compute_morton_bbox / processInternalNode /
calculateBoudingBox compiled for sm_103a, driven by oracle/refkern/refharness.cpp):

  lbvh_<name>.npz   body vertices (thickness already applied), triangles; per-triangle
                    Morton codes and expanded boxes, the de-duplicated sorted codes and
                    triangles, the radix tree's child / parent links (BRTreeNode
                    encoding), leaf boxes, the Morton frame.  Internal boxes are the
                    refit of the reference's own leaves over its own links (the
                    reference's refit kernel has an unfenced read, so its raw boxes are
                    not stored).
  traj_<name>.npz   a cloth (positions, the reference's structure + bend lists), a body,
                    the reference's constants, and the state (x, x_old, contact normal)
                    after 1, 50, 100 and 200 steps of the reference's verlet kernel.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ffi  # noqa: E402
from simulator_gb300 import scenes, springs_from_mesh  # noqa: E402
from simulator_gb300.params import reference_params  # noqa: E402


def host_refit(b):
    ni = len(b["child_a"])
    out = np.zeros((ni, 6), np.float32)
    done = np.zeros(ni, bool)

    def box(c):
        return b["leaf_boxes"][-c - 1] if c < 0 else out[c - 1]

    stack = [0]
    while stack:
        i = stack[-1]
        pend = [c - 1 for c in (b["child_a"][i], b["child_b"][i]) if c > 0 and not done[c - 1]]
        if pend:
            stack += pend
            continue
        stack.pop()
        a, c = box(b["child_a"][i]), box(b["child_b"][i])
        out[i, :3] = np.minimum(np.minimum(np.float32(100.0), a[:3]), c[:3])
        out[i, 3:] = np.maximum(np.maximum(np.float32(-100.0), a[3:]), c[3:])
        done[i] = True
    return out


def soup(n, seed, dup):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-1, 1, size=(n, 3))
    v = c[:, None, :] + rng.normal(0, 0.02, size=(n, 3, 3))
    k = int(dup * n)
    v[rng.choice(n, k, replace=False)] = v[rng.integers(0, n, k)]
    return v.reshape(-1, 3).astype(np.float32), np.arange(3 * n, dtype=np.uint32).reshape(n, 3)


def lbvh_fixture(out_dir, name, xyz, tris):
    cloth = scenes.grid_cloth(4, 1.0, 5.0, pin_top_corners=False)
    cl = springs_from_mesh(cloth.xyz, cloth.faces)
    p = reference_params(2)
    r = ffi.RefSim(p, cloth.xyz, cl, xyz, tris)  # no normals: vertices used as given
    b = r.export_lbvh()
    r.close()
    b["internal_boxes"] = host_refit(b)
    np.savez_compressed(os.path.join(out_dir, f"lbvh_{name}.npz"), body_xyz=xyz, body_tris=tris,
                        box_depth=np.float32(p.box_depth), **{k: v for k, v in b.items() if k != "n_leaves"},
                        n_leaves=np.int64(b["n_leaves"]))


def traj_fixture(out_dir, name, side, subdiv, drop):
    cloth = scenes.grid_cloth(side, 1.0, 0.0, pin_top_corners=False)
    body = scenes.icosphere(subdiv, 0.3, center=(0.0, -drop, 0.0))
    cl = springs_from_mesh(cloth.xyz, cloth.faces)
    p = reference_params(2)
    r = ffi.RefSim(p, cloth.xyz, cl, body.xyz, body.tris, body.normals)
    states = {}
    done = 0
    for k in (1, 50, 100, 200):
        r.step(k - done)
        done = k
        x, xo, n = r.state()
        states[f"x_{k}"], states[f"xo_{k}"], states[f"n_{k}"] = x, xo, n
    r.close()
    np.savez_compressed(os.path.join(out_dir, f"traj_{name}.npz"), cloth_xyz=cloth.xyz,
                        row0=cl[0].row, end0=cl[0].ent["end"], rest0=cl[0].ent["rest"],
                        row1=cl[1].row, end1=cl[1].ent["end"], rest1=cl[1].ent["rest"],
                        body_xyz=body.xyz, body_tris=body.tris, body_normals=body.normals,
                        params=np.frombuffer(bytes(p), np.uint8), **states)


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    ico3 = scenes.icosphere(3, 0.3, (0.1, -0.5, 0.2), noise=0.02, seed=3)
    lbvh_fixture(out_dir, "ico3_noise", ico3.xyz, ico3.tris)
    ico4 = scenes.icosphere(4, 0.3, (0.0, -0.5, 0.0))
    lbvh_fixture(out_dir, "ico4", ico4.xyz, ico4.tris)
    xyz, tris = soup(3000, 11, 0.3)
    lbvh_fixture(out_dir, "soup3000_dup", xyz, tris)
    traj_fixture(out_dir, "sheet24_ico2", 24, 2, 0.31)
    print("written:", sorted(os.listdir(out_dir)))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__)))
