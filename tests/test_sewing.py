"""Seams of multi-piece garments (the reference's SINGLE_LAYER_BOUNDARY springs,
Springs::get_cloth_boundary_spring / get_boundary_boundary_spring, spring.cpp:98-209).

The library's structure list for a sewn garment must equal the plain one plus the
seam springs in the reference's order; the expected seams come from an independent
brute-force restatement (exact nearest neighbours; the inputs are jittered so no two
candidates tie).  The GPU test runs a sewn two-piece garment against the oracle.
"""
import numpy as np
import pytest

import simulator_gb300 as vs
from simulator_gb300 import scenes

F = np.float32


def two_pieces(seed=0, n=8, gap=0.02):
    """Two n x n sheets side by side, a gap apart; each piece's boundary group is a
    copy of its edge column facing the other piece, 4 mm towards it."""
    rng = np.random.default_rng(seed)
    a = scenes.grid_positions(n, 0.4, 0.0) + F([-0.2 - gap / 2, 0, 0])
    b = scenes.grid_positions(n, 0.4, 0.0) + F([0.2 + gap / 2, 0, 0])
    a += rng.normal(0, 1e-4, a.shape).astype(F)
    b += rng.normal(0, 1e-4, b.shape).astype(F)
    ea = a.reshape(n, n, 3)[:, -1] + F([0.004, 0, 0])  # right edge of piece a
    eb = b.reshape(n, n, 3)[:, 0] - F([0.004, 0, 0])   # left edge of piece b
    ea += rng.normal(0, 1e-4, ea.shape).astype(F)
    eb += rng.normal(0, 1e-4, eb.shape).astype(F)
    xyz = np.concatenate([a, ea, b, eb]).astype(F)
    f = scenes.grid_faces(n).astype(np.int64)
    o_b = n * n + n
    faces = np.concatenate([f, f + o_b]).astype(np.uint32)
    return xyz, faces, [n * n, n, n * n, n]


def brute_seams(xyz, groups):
    x64 = xyz.astype(np.float64)
    starts = np.concatenate([[0], np.cumsum(groups)])
    cb, bspans = [], []
    for g in range(0, len(groups), 2):
        piece = np.arange(starts[g], starts[g + 1])
        bnd = np.arange(starts[g + 1], starts[g + 2])
        for v in bnd:
            d = ((x64[piece] - x64[v]) ** 2).sum(1)
            cb.append((int(v), int(piece[np.argmin(d)])))
        bspans.append(bnd)

    def fdist(i, j):
        d = (xyz[j] - xyz[i]).astype(F)
        return np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])

    navg = min(100, len(cb))
    md = F(0)
    for v, c in cb[:navg]:
        md = F(md + fdist(v, c))
    md = F(md / F(navg))
    piece_of = dict(cb)
    seam = set()
    for i, bnd in enumerate(bspans):
        others = np.concatenate([b for j, b in enumerate(bspans) if j != i])
        for v in bnd:
            r = int(others[np.argmin(((x64[others] - x64[v]) ** 2).sum(1))])
            d = fdist(v, r)
            if d < md * F(50) and d > 0:
                seam.add((piece_of[v], piece_of[r]))
    out = []
    for v, c in cb:
        out += [(v, c), (c, v)]
    return out + sorted(seam)


def test_sewn_structure_list_is_faces_plus_seams():
    xyz, faces, groups = two_pieces()
    plain = vs.springs_from_mesh(xyz, faces)
    sewn = vs.springs_from_mesh_sewn(xyz, faces, groups)
    assert np.array_equal(sewn[1].row, plain[1].row) and np.array_equal(sewn[1].ent, plain[1].ent)
    extra = {}
    for a, b in brute_seams(xyz, groups):
        extra.setdefault(a, []).append(b)
    for v in range(len(xyz)):
        p = plain[0].ent["end"][plain[0].row[v]:plain[0].row[v + 1]].tolist()
        s = sewn[0].ent["end"][sewn[0].row[v]:sewn[0].row[v + 1]].tolist()
        assert s == p + extra.get(v, []), v
    # every edge vertex of one piece is sewn to the facing edge vertex of the other
    n = 8
    for k in range(n):
        a_edge, b_edge = k * n + n - 1, n * n + n + k * n
        assert b_edge in sewn[0].ent["end"][sewn[0].row[a_edge]:sewn[0].row[a_edge + 1]]
    rest = sewn[0].ent["rest"]
    assert np.isfinite(rest).all() and (rest > 0).all()


def test_sewing_rejects_bad_groups():
    xyz, faces, groups = two_pieces()
    with pytest.raises(vs.VisgError):
        vs.springs_from_mesh_sewn(xyz, faces, groups[:3])  # odd
    with pytest.raises(vs.VisgError):
        vs.springs_from_mesh_sewn(xyz, faces, [len(xyz), 10])  # more than the mesh


def test_obj_groups(tmp_path):
    p = tmp_path / "g.obj"
    p.write_text("# object piece0\n# 3 vertices\nv 0 0 0\nv 1 0 0\nv 0 1 0\n"
                 "# object piece0_boundary\n# 1 vertices\nv 1 1 0\nf 1 2 3\n")
    assert vs.obj_groups(str(p)).tolist() == [3, 1]


@pytest.mark.gpu
def test_sewn_garment_vs_oracle():
    from oracle.ffi import OracleSim
    xyz, faces, groups = two_pieces(seed=1)
    lists = vs.springs_from_mesh_sewn(xyz, faces, groups)
    body = scenes.icosphere(3, 0.3, (0.0, -0.31, 0.0))
    p = vs.reference_params(2)
    g = vs.Simulator(xyz, lists, body.xyz, body.tris, body.normals, params=p)
    o = OracleSim(p, xyz, lists, body.xyz, body.tris, body.normals, prec=4)
    g.simulate(100)
    o.step(100)
    x, xo, n = g.state()
    ox, oxo, on = (a.astype(F) for a in o.state())
    assert np.array_equal(x, ox) and np.array_equal(xo, oxo) and np.array_equal(n, on)
