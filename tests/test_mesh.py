"""Real-mesh inputs: the OBJ reader (the reference's ObjLoader + Mesh::unified
semantics), the demo's mesh transforms (Mesh::scale / translate / rotation), and
the reference's spring topology built from an OBJ's triangles.

CPU tests check the reader on hand-written files and the transforms against a numpy
float32 restatement; when the reference's own meshes are present on this machine
they are read too (skipped elsewhere).  The GPU test simulates a garment read from
an OBJ file over a body read from another, against the oracle, bit for bit.
"""
import os

import numpy as np
import pytest

import simulator_gb300 as vs
from oracle.build import REFERENCE
from simulator_gb300 import scenes

F = np.float32
REF_RES = os.path.join(REFERENCE, "resources")  # the reference tree the oracle's recipe builds from


def test_obj_reader_forms(tmp_path):
    p = tmp_path / "m.obj"
    p.write_text(
        "# comment\nmtllib x.mtl\n"
        "v 0 0 0\nv 1 0 0\nv 0 1 0\nv 1 1 0 1.0\nv 5 5 5\n"
        "vn 0 0 1\nvn 0 0 -1\nvn 1 0 0\nvn 0 1 0\n"
        "vt 0 0\n"
        "f 1 2 3\n"                  # plain form: normal index = vertex index
        "f 2/1/2 4/1/4 3/1/3 1/1/1\n"  # a quad: the first three corners only
    )
    xyz, nrm, faces = vs.load_obj(str(p))
    assert xyz.shape == (5, 3) and faces.tolist() == [[0, 1, 2], [1, 3, 2]]
    assert np.array_equal(xyz[3], F([1, 1, 0]))
    # vertex 1: normal 2 by the quad's first corner (last corner naming it);
    # vertex 2: normal 3 by the quad's third corner; vertex 0: normal 1 (plain form);
    # vertex 3: normal 4; vertex 4: unused -> 0
    assert np.array_equal(nrm, F([[0, 0, 1], [0, 0, -1], [1, 0, 0], [0, 1, 0], [0, 0, 0]]))
    bad = tmp_path / "bad.obj"
    bad.write_text("v 0 0 0\nf 1 2 3\n")
    with pytest.raises(vs.VisgError):
        vs.load_obj(str(bad))
    with pytest.raises(vs.VisgError):
        vs.load_obj(str(tmp_path / "missing.obj"))


def np_centre(x):
    s = np.zeros(3, F)
    for v in x:
        s = s + v
    return s / F(len(x))


def test_mesh_transforms_match_float32_restatement():
    rng = np.random.default_rng(1)
    x = rng.normal(0, 0.5, (300, 3)).astype(F)
    c = np_centre(x)
    assert np.array_equal(vs.mesh_scale(x.copy(), 3.33), (x - c) * F(3.33))
    assert np.array_equal(vs.mesh_translate(x.copy(), 0.0, 1.98, 0.02), x + F([0.0, 1.98, 0.02]))
    for axis in range(3):
        for deg in (90.0, -4.0):
            a = F(np.float64(F(deg) / F(180)) * 3.1415)
            cs, sn = np.cos(a), np.sin(a)
            m = np.eye(4, dtype=F)  # m[column][row]
            i, j = [(1, 2), (0, 2), (0, 1)][axis]
            m[i][i], m[i][j], m[j][i], m[j][j] = cs, -sn, sn, cs
            v = np.concatenate([x - c, np.ones((len(x), 1), F)], 1)
            want = np.stack([(m[0][r] * v[:, 0] + m[1][r] * v[:, 1]) + (m[2][r] * v[:, 2] + m[3][r] * v[:, 3])
                             for r in range(3)], 1) + c
            got = vs.mesh_rotate(x.copy(), deg, axis)
            assert np.abs(got - want).max() <= 2 * np.spacing(np.abs(want).max()), (axis, deg)


@pytest.mark.skipif(not os.path.isdir(REF_RES), reason="the reference's meshes are not on this machine")
def test_reference_demo_meshes():
    from oracle import ffi
    cloth, cn, cf = vs.load_obj(os.path.join(REF_RES, "cloth/tshirt2/tshirt2.obj"))
    body, bn, bf = vs.load_obj(os.path.join(REF_RES, "pose/female.obj"))
    assert (len(cloth), len(cf), len(body), len(bf)) == (16773, 32589, 6890, 13776)
    assert np.all(np.abs(np.linalg.norm(bn, axis=1) - 1) < 1e-3)  # every body vertex has its OBJ normal
    # the demo's placement (main.cpp:24-32)
    vs.mesh_rotate(cloth, 90, 0)
    vs.mesh_rotate(cloth, -4, 2)
    vs.mesh_scale(cloth, 3.33)
    vs.mesh_translate(cloth, 0, 1.98, 0.02)
    vs.mesh_scale(body, 3.226)
    vs.mesh_translate(body, 0, 1.8, 0)
    assert np.isfinite(cloth).all() and np.isfinite(body).all()
    ours = vs.springs_from_mesh(cloth, cf)
    orc = ffi.springs_from_mesh(cloth, cf)
    for a, b in zip(ours, orc):
        assert np.array_equal(a.row, b.row) and np.array_equal(a.ent, b.ent)
    assert ours[0].n_entries > 3 * len(cf) // 2 and ours[1].n_entries > 0


@pytest.mark.gpu
def test_obj_garment_over_obj_body_vs_oracle(tmp_path):
    from oracle.ffi import OracleSim
    cloth = scenes.grid_cloth(30, 1.0, 0.0)
    body = scenes.icosphere(3, 0.3, (0.0, -0.3, 0.0))
    vs.write_obj(str(tmp_path / "cloth.obj"), cloth.xyz, cloth.faces)
    with open(tmp_path / "body.obj", "w") as f:  # with per-vertex normals, "a/t/n" faces
        for p in body.xyz:
            f.write(f"v {p[0]:.9g} {p[1]:.9g} {p[2]:.9g}\n")
        for nv in body.normals:
            f.write(f"vn {nv[0]:.9g} {nv[1]:.9g} {nv[2]:.9g}\n")
        for t in body.tris.astype(np.int64) + 1:
            f.write(f"f {t[0]}/1/{t[0]} {t[1]}/1/{t[1]} {t[2]}/1/{t[2]}\n")
    cx, _, cf = vs.load_obj(str(tmp_path / "cloth.obj"))
    bx, bn, bf = vs.load_obj(str(tmp_path / "body.obj"))
    assert np.array_equal(cf, cloth.faces) and np.array_equal(bf, body.tris)
    lists = vs.springs_from_mesh(cx, cf)
    p = vs.reference_params(2)
    g = vs.Simulator(cx, lists, bx, bf, bn, params=p)
    o = OracleSim(p, cx, lists, bx, bf, bn, prec=4)
    g.set_faces(cf)
    g.simulate(80)
    o.step(80)
    x, xo, n = g.state()
    ox, oxo, on = (a.astype(F) for a in o.state())
    assert np.array_equal(x, ox) and np.array_equal(xo, oxo) and np.array_equal(n, on)
    assert g.count_contacts() > 0
    pos4, vn, fn = g.render()
    assert np.array_equal(pos4[:, :3], x) and np.isfinite(vn).all() and len(fn) == len(cf)


def test_obj_reader_empty_parts(tmp_path):
    """Files without groups, faces or vertices read as empty parts (the copies of
    empty arrays touch nothing), or are rejected with an error."""
    p = tmp_path / "nogroups.obj"
    p.write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    assert vs.obj_groups(str(p)).tolist() == []
    p = tmp_path / "nofaces.obj"
    p.write_text("v 0 0 0\nv 1 0 0\n")
    xyz, nrm, faces = vs.load_obj(str(p))
    assert xyz.shape == (2, 3) and faces.shape == (0, 3)
    p = tmp_path / "empty.obj"
    p.write_text("# nothing here\n")
    try:
        xyz, nrm, faces = vs.load_obj(str(p))
        assert len(xyz) == 0 and len(faces) == 0
    except vs.VisgError:
        pass
