"""The output stage of a step (the reference's cuda_update_vbo, headless): positions
as (x, y, z, 1), face normals of the positions the step started from, vertex normals
as the normalised sum of each vertex's face normals in face order.

CPU: the oracle against an independent numpy float32 restatement (bit for bit).
GPU: the library against the oracle and against the reference's own kernels
(update_vbo_pos, compute_face_normal, compute_vbo_normal), bit for bit.
"""
import numpy as np
import pytest

from oracle import ffi
from oracle.ffi import OracleSim
from simulator_gb300 import scenes

F = np.float32


def np_render(x, xp, faces):
    """float32, one rounding per operation, GLM 0.9.9.8's cross / normalize."""
    def cross(a, b):
        return np.stack([a[:, 1] * b[:, 2] - b[:, 1] * a[:, 2], a[:, 2] * b[:, 0] - b[:, 2] * a[:, 0],
                         a[:, 0] * b[:, 1] - b[:, 0] * a[:, 1]], 1)

    def normalize(v):
        d = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
        return v * (F(1) / np.sqrt(d))[:, None]

    x, xp = x.astype(F), xp.astype(F)
    p0, p1, p2 = xp[faces[:, 0]], xp[faces[:, 1]], xp[faces[:, 2]]
    fn = normalize(cross(p1 - p0, p2 - p0))
    acc = np.zeros_like(x)
    order = np.argsort(np.repeat(np.arange(len(faces)), 3), kind="stable")  # faces in order, per vertex
    for k in order:
        f, v = divmod(int(k), 3)
        acc[faces[f, v]] = acc[faces[f, v]] + fn[f]
    with np.errstate(invalid="ignore", divide="ignore"):
        vn = normalize(acc)
    pos4 = np.concatenate([x, np.ones((len(x), 1), F)], 1)
    return pos4, vn, fn


def same(a, b):
    return np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_oracle_render_matches_float32_restatement():
    rng = np.random.default_rng(4)
    cloth = scenes.grid_cloth(17, 1.0, 0.0, jitter=1e-3, seed=2)
    faces = cloth.faces.astype(np.uint32)
    x = cloth.xyz + rng.normal(0, 2e-3, cloth.xyz.shape).astype(F)
    xp = cloth.xyz
    with np.errstate(invalid="ignore", divide="ignore"):
        want = np_render(x, xp, faces)
    got = ffi.render(x, xp, faces)
    for g, w in zip(got, want):
        assert same(g, w)
    # a vertex without faces gets normalize(0): NaN, as in the reference
    x2 = np.concatenate([x, [[0.0, 1.0, 0.0]]]).astype(F)
    _, vn, _ = ffi.render(x2, np.concatenate([xp, [[0.0, 1.0, 0.0]]]).astype(F), faces)
    assert np.isnan(vn[-1]).all() and np.isfinite(vn[:-1]).all()


def draped():
    cloth = scenes.grid_cloth(40, 1.0, 0.0)
    body = scenes.icosphere(3, 0.3, (0.0, -0.3, 0.0))  # with the 5 mm push, 5 mm into the sheet
    return cloth, body, scenes.physics_params(2)


@pytest.mark.gpu
def test_render_matches_oracle_and_reference_kernels():
    import simulator_gb300 as vs
    cloth, body, p = draped()
    faces = cloth.faces.astype(np.uint32)
    g = vs.Simulator(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, params=p, pinned=cloth.pinned)
    o = OracleSim(p, cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, prec=4, pinned=cloth.pinned)
    g.set_faces(faces)
    g.simulate(119)
    o.step(119)
    xp = o.state()[0].astype(F)
    g.simulate(1)
    o.step(1)
    x = o.state()[0].astype(F)
    assert g.count_contacts() > 0  # the step projected vertices: x_old differs from the pre-step x
    want = ffi.render(x, xp, faces)
    got = g.render(normals_of_previous=True)
    for a, b in zip(got, want):
        assert same(a, b)
    cur = g.render(normals_of_previous=False)  # normals of the current positions
    want_cur = ffi.render(x, x, faces)
    for a, b in zip(cur, want_cur):
        assert same(a, b)
    if ffi.refkern_available():
        ref = ffi.ref_render(x, xp, faces)
        for a, b in zip(got, ref):
            assert same(a, b)


@pytest.mark.gpu
def test_batch_render_equals_per_garment():
    import simulator_gb300 as vs
    p = scenes.physics_params(2)
    items = []
    for side in (9, 16, 12):
        cloth = scenes.grid_cloth(side, 1.0, 0.0)
        body = scenes.icosphere(2, 0.3, (0.0, -0.31, 0.0))
        items.append((cloth, body))
    b = vs.BatchSimulator(p)
    for cloth, body in items:
        b.add(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, pinned=cloth.pinned)
    b.finalize()
    for gi, (cloth, _) in enumerate(items):
        b.set_faces(gi, cloth.faces)
    b.step(40)
    pos4, vn, fn = b.render()
    f0 = 0
    for gi, (cloth, body) in enumerate(items):
        s = vs.Simulator(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, params=p, pinned=cloth.pinned)
        s.set_faces(cloth.faces)
        s.simulate(40)
        q4, qn, qf = s.render()
        sl = slice(int(b.offsets[gi]), int(b.offsets[gi + 1]))
        assert same(pos4[sl], q4) and same(vn[sl], qn)
        assert same(fn[f0:f0 + len(qf)], qf)
        f0 += len(qf)


@pytest.mark.gpu
def test_render_requires_faces_for_normals():
    import simulator_gb300 as vs
    cloth, body, p = draped()
    g = vs.Simulator(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, params=p)
    with pytest.raises(vs.VisgError):
        g.render()
    with pytest.raises(vs.VisgError):
        g.set_faces(np.array([[0, 1, len(cloth.xyz)]], np.uint32))


def np_sh(normals, rgb):
    """The SH fragment shader (sh.frag:13-55), float32, term by term in its order."""
    C1, C2, C3, C4, C5 = F(0.429043), F(0.511664), F(0.743125), F(0.886227), F(0.247708)
    L = {k: np.array(v, F) for k, v in dict(L00=(0.87, 0.87, 0.86), L1m1=(0.17, 0.24, 0.31), L10=(0.03, 0.03, 0.03),
                                            L11=(-0.004, -0.03, -0.05), L2m2=(-0.12, -0.12, -0.11),
                                            L2m1=(0.003, 0.003, 0.007), L20=(-0.03, -0.02, -0.02),
                                            L21=(-0.08, -0.08, -0.09), L22=(-0.16, -0.19, -0.22)).items()}
    n = normals.astype(F)
    d = (n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2]
    t = n * (F(1) / np.sqrt(d))[:, None]
    x, y, z = t[:, :1], t[:, 1:2], t[:, 2:3]
    a, b = F(2) * C1, F(2) * C2
    r = (C1 * L["L22"]) * (x * x - y * y)
    r = r + ((C3 * L["L20"]) * z) * z
    r = r + C4 * L["L00"]
    r = r - C5 * L["L20"]
    r = r + ((a * L["L2m2"]) * x) * y
    r = r + ((a * L["L21"]) * x) * y
    r = r + ((a * L["L2m1"]) * y) * z
    r = r + (b * L["L11"]) * x
    r = r + (b * L["L1m1"]) * y
    r = r + (b * L["L10"]) * z
    r = (F(0) + r * F(1)) + F(0)
    return r * np.asarray(rgb, F)


def test_oracle_sh_shade_matches_float32_restatement():
    rng = np.random.default_rng(9)
    nrm = rng.normal(0, 1, (500, 3)).astype(F)
    rgb = F([0.9, 0.7, 0.5])
    assert same(ffi.sh_shade(nrm, rgb), np_sh(nrm, rgb))


@pytest.mark.gpu
def test_render_shaded_matches_oracle():
    import simulator_gb300 as vs
    cloth, body, p = draped()
    g = vs.Simulator(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, params=p, pinned=cloth.pinned)
    g.set_faces(cloth.faces)
    g.simulate(30)
    rgb = (0.8, 0.6, 0.4)
    pos4, vn, col = g.render_shaded(rgb)
    q4, qn, _ = g.render()
    assert same(pos4, q4) and same(vn, qn)
    assert same(col, ffi.sh_shade(vn, rgb))
