"""Shared scene builders and comparisons for the tests."""
import numpy as np

from simulator_gb300 import scenes
from simulator_gb300.params import reference_params

LBVH_INT_KEYS = ("tri_codes", "sorted_codes", "sorted_tris", "child_a", "child_b", "parent_internal", "parent_leaf")
LBVH_BOX_KEYS = ("tri_boxes", "internal_boxes", "leaf_boxes", "root_box")


def lbvh_diff(a: dict, b: dict) -> list:
    """Names of the fields that differ (integers bit-exact, boxes by value)."""
    bad = []
    if a["n_leaves"] != b["n_leaves"]:
        return ["n_leaves"]
    for k in LBVH_INT_KEYS:
        if not np.array_equal(a[k], b[k]):
            bad.append(k)
    for k in LBVH_BOX_KEYS:
        if not np.array_equal(a[k], b[k]):  # == treats -0 and +0 as equal
            bad.append(k)
    return bad


def soup(n_tris: int, seed: int, spread: float = 1.0, dup_frac: float = 0.0):
    """Random triangle soup; dup_frac of the triangles are copies (duplicate codes)."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-spread, spread, size=(n_tris, 3))
    v = c[:, None, :] + rng.normal(0, 0.02 * spread, size=(n_tris, 3, 3))
    ndup = int(dup_frac * n_tris)
    if ndup:
        src = rng.integers(0, n_tris, size=ndup)
        dst = rng.choice(n_tris, size=ndup, replace=False)
        v[dst] = v[src]
    xyz = v.reshape(-1, 3).astype(np.float32)
    tris = np.arange(3 * n_tris, dtype=np.uint32).reshape(n_tris, 3)
    return xyz, tris


def ref_scene(side=24, subdiv=2, radius=0.3, drop=0.31, lists="grid"):
    """Sheet above an icosphere with the reference's constants; lists = 'grid'
    (3 families) or 'mesh' (the reference's structure + bend lists)."""
    cloth = scenes.grid_cloth(side, 1.0, 0.0, pin_top_corners=False)
    body = scenes.icosphere(subdiv, radius, center=(0.0, -drop, 0.0))
    if lists == "mesh":
        from simulator_gb300 import springs_from_mesh
        cl = springs_from_mesh(cloth.xyz, cloth.faces)
        p = reference_params(2)
    else:
        cl = cloth.lists
        p = reference_params(3)
        p.list_k[:] = (100.0, 60.0, 2.0, 0.0)
    return cloth, cl, body, p


def config_params(substeps=2, **kw):
    return scenes.physics_params(substeps, **kw)
