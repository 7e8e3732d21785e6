"""CPU tests: the oracle's own consistency, the host logic of the library and its
C ABI (loaded without a GPU), and the bottom-up radix-tree construction the
device build uses, restated in Python and checked against the oracle's Karras
construction (cudaBRT.cu:120-161)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT, has_gpu
from helpers import lbvh_diff, ref_scene, soup
from oracle.ffi import OracleSim, springs_from_mesh as orc_springs
from simulator_gb300 import scenes
from simulator_gb300.params import reference_params


def oracle_body(xyz, tris, prec=4):
    cloth = scenes.grid_cloth(4, 1.0, 0.0, pin_top_corners=False)
    p = reference_params(3)
    return OracleSim(p, cloth.xyz, cloth.lists, xyz, tris, None, prec=prec)


def check_tree(b):
    """Structural invariants of a binary radix tree in the reference layout."""
    n = b["n_leaves"]
    codes = b["sorted_codes"]
    assert np.all(np.diff(codes.astype(np.int64)) > 0), "codes sorted and distinct"
    if n < 2:
        return
    ca, cb = b["child_a"], b["child_b"]
    kids = np.concatenate([ca, cb])
    assert sorted((-kids[kids < 0] - 1).tolist()) == list(range(n))
    assert sorted((kids[kids > 0] - 1).tolist()) == list(range(1, n - 1))
    assert b["parent_internal"][0] == 0
    for i in range(n - 1):
        for c in (ca[i], cb[i]):
            if c < 0:
                assert b["parent_leaf"][-c - 1] == i + 1
                box = b["leaf_boxes"][-c - 1]
            else:
                assert b["parent_internal"][c - 1] == i + 1
                box = b["internal_boxes"][c - 1]
            assert np.all(b["internal_boxes"][i][:3] <= box[:3]) and np.all(b["internal_boxes"][i][3:] >= box[3:])


@pytest.mark.parametrize("subdiv", [0, 1, 2, 3, 4])
def test_oracle_lbvh_icosphere_valid(subdiv):
    body = scenes.icosphere(subdiv, 0.3, center=(0.1, -0.4, 0.05), noise=0.02, seed=subdiv)
    b = oracle_body(body.xyz, body.tris).export_lbvh()
    check_tree(b)
    # leaf boxes are the expanded boxes of the sorted triangles
    assert np.array_equal(b["leaf_boxes"], b["tri_boxes"][b["sorted_tris"]])


@pytest.mark.parametrize("n,dup", [(2, 0.0), (3, 0.0), (127, 0.0), (128, 0.0), (129, 0.0), (1000, 0.3), (4096, 0.5)])
def test_oracle_lbvh_dedupe_keeps_lowest_index(n, dup):
    xyz, tris = soup(n, seed=n, dup_frac=dup)
    b = oracle_body(xyz, tris).export_lbvh()
    check_tree(b)
    codes = b["tri_codes"]
    order = np.lexsort((np.arange(n), codes))  # (code, triangle) order
    first = order[np.concatenate([[True], codes[order][1:] != codes[order][:-1]])]
    assert np.array_equal(b["sorted_tris"], first)
    assert np.array_equal(b["sorted_codes"], codes[first])


def bottom_up_build(codes: np.ndarray, seed: int = 0):
    """The device build's chunk climb (visg_lbvh.cu build_chunk), executed leaf by
    leaf in a random order: climb while the parent has already been reached by the
    other child.
    Returns (links A/B per split node, ranges, root split)."""
    n = len(codes)
    rng = np.random.default_rng(seed)

    def delta(i, j):
        if j < 0 or j >= n:
            return -1
        x = int(codes[i]) ^ int(codes[j])
        return 32 - x.bit_length()

    la = np.zeros(n - 1, np.int64)
    lb = np.zeros(n - 1, np.int64)
    rng_l = np.zeros(n - 1, np.int64)
    rng_r = np.zeros(n - 1, np.int64)
    flag = np.zeros(n - 1, np.int64)
    root = -1
    for i in rng.permutation(n):
        l = r = int(i)
        link = ~int(i)
        while True:
            if delta(r, r + 1) > delta(l, l - 1):
                g = r
                la[g] = link
                rng_l[g] = l
            else:
                g = l - 1
                lb[g] = link
                rng_r[g] = r
            flag[g] += 1
            if flag[g] == 1:
                break
            l, r = int(rng_l[g]), int(rng_r[g])
            link = g
            if l == 0 and r == n - 1:
                root = g
                break
    return la, lb, rng_l, rng_r, root


def renumber(la, lb, rl, rr, root):
    """visg_export_lbvh's renumbering into the reference layout."""
    ni = len(la)
    k = np.full(ni, -1, np.int64)
    k[root] = 0
    for g in range(ni):
        if la[g] >= 0:
            k[la[g]] = rr[la[g]]
        if lb[g] >= 0:
            k[lb[g]] = rl[lb[g]]
    ca = np.zeros(ni, np.int64)
    cb = np.zeros(ni, np.int64)
    for g in range(ni):
        ca[k[g]] = -(~la[g]) - 1 if la[g] < 0 else k[la[g]] + 1
        cb[k[g]] = -(~lb[g]) - 1 if lb[g] < 0 else k[lb[g]] + 1
    return ca, cb


@pytest.mark.parametrize("n,seed", [(2, 0), (3, 1), (17, 2), (256, 3), (1000, 4), (3001, 5)])
def test_bottom_up_build_equals_karras(n, seed):
    xyz, tris = soup(n, seed=seed, dup_frac=0.1)
    b = oracle_body(xyz, tris).export_lbvh()
    codes = b["sorted_codes"]
    if len(codes) < 2:
        pytest.skip("fewer than two distinct codes")
    for order_seed in range(3):
        la, lb, rl, rr, root = bottom_up_build(codes, order_seed)
        assert rl[root] == 0 and rr[root] == len(codes) - 1
        ca, cb = renumber(la, lb, rl, rr, root)
        assert np.array_equal(ca, b["child_a"]) and np.array_equal(cb, b["child_b"])


def incremental_merge(old_codes: np.ndarray, new_codes: np.ndarray) -> np.ndarray:
    """The rebuild's merge path (visg_lbvh.cu phase_merge), restated: the last build's
    list sorted by (old code, triangle), the triangles whose code changed sorted by
    (new code, triangle) and by (old code, triangle), and each entry's new position
    from lower bounds into those two arrays.  Returns the keys (code << 32 |
    triangle) by position, each position written once."""
    nt = len(old_codes)
    tri = np.arange(nt, dtype=np.uint64)
    old_list = np.sort((old_codes.astype(np.uint64) << np.uint64(32)) | tri)
    chg = np.nonzero(new_codes != old_codes)[0]
    nc = len(chg)
    knew = np.sort((new_codes[chg].astype(np.uint64) << np.uint64(32)) | tri[chg])
    kold = np.sort((old_codes[chg].astype(np.uint64) << np.uint64(32)) | tri[chg])
    below = lambda a, x: int(np.searchsorted(a, x, side="left"))  # entries of a below x
    out = np.zeros(nt, np.uint64)
    hits = np.zeros(nt, np.int64)
    for j in range(below(knew, old_list[0])):  # changed entries below the first old key
        out[j] = knew[j]
        hits[j] += 1
    for s in range(nt):
        ks = old_list[s]
        q, r = below(kold, ks), below(knew, ks)
        if not (q < nc and kold[q] == ks):  # unchanged: keeps its place among the others
            out[s - q + r] = ks
            hits[s - q + r] += 1
        r1, q1 = (below(knew, old_list[s + 1]), below(kold, old_list[s + 1])) if s + 1 < nt else (nc, nc)
        for j in range(r, r1):  # changed entries between old slots s and s + 1
            out[j + s + 1 - q1] = knew[j]
            hits[j + s + 1 - q1] += 1
    assert (hits == 1).all()
    return out


@pytest.mark.parametrize("seed", range(6))
def test_incremental_merge_equals_a_full_sort(seed):
    """The merge that replaces the radix sort when few Morton codes changed gives the
    stable (code, triangle) order of the new codes: random code sets with many
    duplicates, with none, some and all of the codes changed."""
    rng = np.random.default_rng(seed)
    for _ in range(100):
        nt = int(rng.integers(1, 80))
        old = rng.integers(0, int(rng.integers(1, 40)), nt).astype(np.uint32)
        new = old.copy()
        k = int(rng.integers(0, nt + 1)) if rng.random() < 0.8 else nt
        idx = rng.choice(nt, size=k, replace=False)
        new[idx] = rng.integers(0, 40, k).astype(np.uint32)
        tri = np.arange(nt, dtype=np.uint64)
        full = np.sort((new.astype(np.uint64) << np.uint64(32)) | tri)
        assert np.array_equal(incremental_merge(old, new), full)


def test_query_matches_manual_first_hit():
    body = scenes.icosphere(2, 0.3, center=(0.0, 0.0, 0.0))
    s = oracle_body(body.xyz, body.tris)
    b = s.export_lbvh()
    rng = np.random.default_rng(0)
    pts = rng.uniform(-0.35, 0.35, size=(2000, 3)).astype(np.float32)
    leaf, inside, dist, nrm = s.query(pts)

    def inb(p, box):
        return np.all(p >= box[:3]) and np.all(p <= box[3:])

    def first_hit(p):
        stack = [None]
        node = 0
        while node is not None:
            a, c = b["child_a"][node], b["child_b"][node]
            ba = b["leaf_boxes"][-a - 1] if a < 0 else b["internal_boxes"][a - 1]
            bb = b["leaf_boxes"][-c - 1] if c < 0 else b["internal_boxes"][c - 1]
            ol, orr = inb(p, ba), inb(p, bb)
            if ol and a < 0:
                return -a - 1
            if orr and c < 0:
                return -c - 1
            tl, tr = ol and a > 0, orr and c > 0
            if not tl and not tr:
                node = stack.pop()
            else:
                node = a - 1 if tl else c - 1
                if tl and tr:
                    stack.append(c - 1)
        return -1

    for i in range(0, 2000, 7):
        assert leaf[i] == first_hit(pts[i])
    assert inside.sum() > 0


def test_fp32_oracle_tracks_fp64():
    cloth, lists, body, p = ref_scene(side=16, subdiv=2)
    a = OracleSim(p, cloth.xyz, lists, body.xyz, body.tris, body.normals, prec=4)
    b = OracleSim(p, cloth.xyz, lists, body.xyz, body.tris, body.normals, prec=8)
    a.step(30)
    b.step(30)
    xa, _, _ = a.state()
    xb, _, _ = b.state()
    assert np.abs(xa - xb).max() < 1e-4


def test_fp64_adjoint_matches_finite_differences():
    """FP64 oracle adjoint vs central differences (no contacts: body far away)."""
    cloth = scenes.grid_cloth(6, 0.3, 0.0, pin_top_corners=True)
    p = scenes.physics_params(4)
    rng = np.random.default_rng(1)
    lists = []
    for sl in cloth.lists:
        lists.append(scenes.SpringList(sl.row, sl.ent, (p.list_k[len(lists)] * np.exp(rng.normal(0, 0.2, sl.n_entries))).astype(np.float32)))
    steps = 20
    target = cloth.xyz + 0.01

    def loss(lst):
        s = OracleSim(p, cloth.xyz, lst, prec=8, pinned=cloth.pinned)
        s.step(steps)
        x, _, _ = s.state()
        return float(((x - target) ** 2).sum() / len(x))

    s = OracleSim(p, cloth.xyz, lists, prec=8, pinned=cloth.pinned)
    s.forward(steps)
    x, _, _ = s.state()
    dk, ds = s.backward(2.0 * (x - target) / len(x))
    off = np.concatenate([[0], np.cumsum([sl.n_entries for sl in lists])])
    for l, e in [(0, 3), (1, 5), (2, 7), (0, 20)]:
        h = 1e-3
        kp = [sl.k.astype(np.float64).copy() for sl in lists]
        base = kp[l][e]
        # per-entry stiffness is stored as float32: perturb by an exactly representable step
        up = [scenes.SpringList(sl.row, sl.ent, k.astype(np.float32)) for sl, k in zip(lists, kp)]
        up[l].k[e] = np.float32(base + h)
        dn = [scenes.SpringList(sl.row, sl.ent, k.astype(np.float32)) for sl, k in zip(lists, kp)]
        dn[l].k[e] = np.float32(base - h)
        hh = (float(up[l].k[e]) - float(dn[l].k[e])) / 2
        fd = (loss(up) - loss(dn)) / (2 * hh)
        g = dk[off[l] + e]
        assert abs(g - fd) <= 1e-3 * max(abs(fd), 1e-8), (l, e, g, fd)


def _header_symbols():
    text = open(os.path.join(ROOT, "include", "visg_sim.h")).read()
    return sorted(set(re.findall(r"\b(visg_\w+)\s*\(", text)))


def test_library_exports_every_header_symbol():
    import simulator_gb300 as vs
    L = C.CDLL(vs.LIB_PATH)
    syms = _header_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_library_version_and_defaults():
    import simulator_gb300 as vs
    L = vs.lib()
    assert b"sm_103a" in L.visg_version()
    p = vs.VisgParams()
    L.visg_default_params(C.byref(p))
    r = reference_params(2)
    for f, _ in vs.VisgParams._fields_:
        a, b = getattr(p, f), getattr(r, f)
        if hasattr(a, "__len__"):
            assert list(a)[: len(b)] == list(b)[: len(a)], f
        else:
            assert a == b, f


@pytest.mark.skipif(has_gpu(), reason="checks the no-device error path")
def test_create_without_gpu_fails_loudly():
    import simulator_gb300 as vs
    cloth = scenes.grid_cloth(4)
    with pytest.raises(vs.VisgError) as e:
        vs.Simulator(cloth.xyz, cloth.lists, params=reference_params(3))
    assert e.value.code == -4


@pytest.mark.parametrize("side", [3, 8, 17])
def test_springs_from_mesh_matches_oracle(side):
    import simulator_gb300 as vs
    cloth = scenes.grid_cloth(side)
    a = vs.springs_from_mesh(cloth.xyz, cloth.faces)
    b = orc_springs(cloth.xyz, cloth.faces)
    for x, y in zip(a, b):
        assert np.array_equal(x.row, y.row)
        assert np.array_equal(x.ent["end"], y.ent["end"])
        assert np.array_equal(x.ent["rest"], y.ent["rest"])
    # structure list of a triangulated grid: row/col/one diagonal neighbours
    assert a[0].n_entries == 2 * (2 * side * (side - 1) + (side - 1) ** 2)


def test_springs_from_icosphere_bend_pairs():
    import simulator_gb300 as vs
    body = scenes.icosphere(1)
    a = vs.springs_from_mesh(body.xyz, body.tris)
    b = orc_springs(body.xyz, body.tris)
    assert np.array_equal(a[1].ent["end"], b[1].ent["end"])
    # closed manifold: every edge is shared by two faces -> one bend pair per edge
    assert a[1].n_entries == 2 * (3 * len(body.tris) // 2)


def test_grid_spring_counts():
    c = scenes.grid_cloth(64)
    assert [sl.n_entries // 2 for sl in c.lists] == [8064, 7938, 7936]
    c = scenes.grid_cloth(512)
    assert sum(sl.n_entries for sl in c.lists) == 3_135_492


def test_icosphere_counts_and_orientation():
    for s, (v, t) in {4: (2562, 5120), 7: (163842, 327680)}.items():
        b = scenes.icosphere(s, 0.3)
        assert (len(b.xyz), len(b.tris)) == (v, t)
    b = scenes.icosphere(3, 1.0)
    tri = b.xyz[b.tris]
    n = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    assert np.all((n * tri.mean(1)).sum(1) > 0), "outward winding"


def test_capsules_outward():
    b = scenes.three_capsules()
    assert 19000 < len(b.tris) < 21000
