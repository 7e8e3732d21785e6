"""Seeded synthetic cloth/body scenes with the shapes of the benchmark workloads.

Everything here builds host-side numpy inputs for the simulator; nothing runs on
the GPU.  Meshes follow the reference's conventions (src/Mesh.h, src/ObjLoader.h):
float32 xyz vertex arrays, uint32 triangle index triples wound counter-clockwise
seen from outside, so that normalize(cross(v1 - v0, v2 - v0)) is the outward
normal that the expanded boxes and the point/plane test assume
(src/bvh/primitive.cu:79-91,110-125).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

SPRING_DTYPE = np.dtype([("end", "<i4"), ("rest", "<f4")])  # == VisgSpring / s_spring


@dataclass
class SpringList:
    """One CSR spring list: row offsets (n+1) and entries (end, rest)."""

    row: np.ndarray
    ent: np.ndarray
    k: np.ndarray | None = None  # optional per-entry stiffness

    @property
    def n_entries(self) -> int:
        return int(self.row[-1])


@dataclass
class Cloth:
    xyz: np.ndarray  # (n, 3) float32
    lists: list[SpringList]
    faces: np.ndarray | None = None  # (f, 3) uint32, for normals / rendering
    pinned: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint32))
    side: int = 0


@dataclass
class Body:
    xyz: np.ndarray  # (v, 3) float32
    tris: np.ndarray  # (t, 3) uint32
    normals: np.ndarray | None = None  # (v, 3) float32 per-vertex normals


# --------------------------------------------------------------------------------------
# cloth
# --------------------------------------------------------------------------------------
def grid_positions(n: int, side: float = 1.0, height: float = 0.0, jitter: float = 0.0,
                   seed: int | None = None) -> np.ndarray:
    """n x n vertices in the y = height plane, centred on the y axis, row-major
    (vertex r*n + c at x = c*h - side/2, z = r*h - side/2)."""
    h = side / (n - 1)
    c, r = np.meshgrid(np.arange(n), np.arange(n))
    x = c.ravel() * h - side / 2.0
    z = r.ravel() * h - side / 2.0
    p = np.stack([x, np.full(n * n, height), z], axis=1)
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        p = p + rng.normal(0.0, jitter, size=p.shape)
    return np.ascontiguousarray(p, dtype=np.float32)


def _csr_from_pairs(n_vertices: int, src: np.ndarray, dst: np.ndarray, xyz: np.ndarray) -> SpringList:
    """Directed entries src->dst grouped by src, ascending dst within a row;
    rest length = initial distance (spring.cpp:386)."""
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    row = np.zeros(n_vertices + 1, np.uint32)
    np.add.at(row, src + 1, 1)
    row = np.cumsum(row, dtype=np.uint64).astype(np.uint32)
    ent = np.zeros(len(src), SPRING_DTYPE)
    ent["end"] = dst
    d = xyz[dst].astype(np.float32) - xyz[src].astype(np.float32)
    ent["rest"] = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]).astype(np.float32)
    return SpringList(row=row, ent=ent)


def grid_spring_lists(n: int, xyz: np.ndarray) -> list[SpringList]:
    """The three spring families of an n x n grid as three CSR lists:
    structural (1 apart along rows/columns), shear (both diagonals), bend (2 apart)."""
    idx = np.arange(n * n).reshape(n, n)

    def both(a, b):
        a, b = a.ravel(), b.ravel()
        return np.concatenate([a, b]), np.concatenate([b, a])

    fam = []
    s = [both(idx[:, :-1], idx[:, 1:]), both(idx[:-1, :], idx[1:, :])]
    fam.append((np.concatenate([x[0] for x in s]), np.concatenate([x[1] for x in s])))
    s = [both(idx[:-1, :-1], idx[1:, 1:]), both(idx[:-1, 1:], idx[1:, :-1])]
    fam.append((np.concatenate([x[0] for x in s]), np.concatenate([x[1] for x in s])))
    s = [both(idx[:, :-2], idx[:, 2:]), both(idx[:-2, :], idx[2:, :])]
    fam.append((np.concatenate([x[0] for x in s]), np.concatenate([x[1] for x in s])))
    return [_csr_from_pairs(n * n, a, b, xyz) for a, b in fam]


def grid_faces(n: int) -> np.ndarray:
    """Two triangles per grid cell, wound so the normal points to +y."""
    idx = np.arange(n * n).reshape(n, n)
    a, b = idx[:-1, :-1].ravel(), idx[:-1, 1:].ravel()
    c, d = idx[1:, :-1].ravel(), idx[1:, 1:].ravel()
    f = np.concatenate([np.stack([a, c, b], 1), np.stack([b, c, d], 1)])
    return np.ascontiguousarray(f, dtype=np.uint32)


def grid_cloth(n: int, side: float = 1.0, height: float = 0.0, jitter: float = 0.0,
               seed: int | None = None, pin_top_corners: bool = True) -> Cloth:
    xyz = grid_positions(n, side, height, jitter, seed)
    pins = np.array([0, n - 1], np.uint32) if pin_top_corners else np.zeros(0, np.uint32)
    return Cloth(xyz=xyz, lists=grid_spring_lists(n, xyz), faces=grid_faces(n), pinned=pins, side=n)


# --------------------------------------------------------------------------------------
# bodies
# --------------------------------------------------------------------------------------
_PHI = (1.0 + 5.0 ** 0.5) / 2.0
_ICO_V = np.array([[-1, _PHI, 0], [1, _PHI, 0], [-1, -_PHI, 0], [1, -_PHI, 0],
                   [0, -1, _PHI], [0, 1, _PHI], [0, -1, -_PHI], [0, 1, -_PHI],
                   [_PHI, 0, -1], [_PHI, 0, 1], [-_PHI, 0, -1], [-_PHI, 0, 1]], np.float64)
_ICO_F = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                   [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                   [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                   [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], np.int64)


def icosphere(subdiv: int, radius: float = 1.0, center=(0.0, 0.0, 0.0), noise: float = 0.0,
              seed: int | None = None) -> Body:
    """Geodesic sphere: 10*4^s + 2 vertices, 20*4^s triangles.  `noise` perturbs
    each vertex radius by a factor U(1 - noise, 1 + noise); normals stay radial."""
    v = _ICO_V / np.linalg.norm(_ICO_V, axis=1, keepdims=True)
    f = _ICO_F.copy()
    for _ in range(subdiv):
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        e.sort(axis=1)
        uniq, inv = np.unique(e, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = len(v)
        v = np.concatenate([v, mid])
        nf = len(f)
        ab, bc, ca = inv[:nf] + base, inv[nf:2 * nf] + base, inv[2 * nf:] + base
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        f = np.concatenate([np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
                            np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1)])
    nrm = v.copy()
    r = np.full(len(v), radius)
    if noise > 0.0:
        rng = np.random.default_rng(seed)
        r = r * rng.uniform(1.0 - noise, 1.0 + noise, size=len(v))
    xyz = v * r[:, None] + np.asarray(center, np.float64)[None, :]
    return Body(xyz=np.ascontiguousarray(xyz, np.float32), tris=np.ascontiguousarray(f, np.uint32),
                normals=np.ascontiguousarray(nrm, np.float32))


def capsule(p0, p1, radius: float, n_around: int, n_rings: int) -> Body:
    """Closed capsule around the segment p0-p1: hemispherical caps (n_rings/2 rings
    each, poles excluded) joined by a cylinder; outward-wound triangles."""
    p0, p1 = np.asarray(p0, np.float64), np.asarray(p1, np.float64)
    axis = p1 - p0
    length = np.linalg.norm(axis)
    w = axis / length
    tmp = np.array([1.0, 0.0, 0.0]) if abs(w[0]) < 0.9 else np.array([0.0, 1.0, 0.0])
    u = np.cross(w, tmp)
    u /= np.linalg.norm(u)
    vv = np.cross(w, u)
    half = n_rings // 2
    # latitude from -pi/2 (p0 pole) to +pi/2 (p1 pole); rings exclude the poles
    lat = np.concatenate([np.linspace(-np.pi / 2, 0.0, half + 1)[1:], np.linspace(0.0, np.pi / 2, half + 1)[:-1]])
    ang = np.linspace(0.0, 2 * np.pi, n_around, endpoint=False)
    verts, norms = [], []
    for k, phi in enumerate(lat):
        c = p0 if k < half else p1
        ring_n = (np.cos(phi) * (np.cos(ang)[:, None] * u[None, :] + np.sin(ang)[:, None] * vv[None, :])
                  + np.sin(phi) * w[None, :])
        verts.append(c[None, :] + radius * ring_n)
        norms.append(ring_n)
    verts.append((p0 - radius * w)[None, :]); norms.append(-w[None, :])
    verts.append((p1 + radius * w)[None, :]); norms.append(w[None, :])
    xyz = np.concatenate(verts)
    nrm = np.concatenate(norms)
    R = len(lat)
    bot, top = R * n_around, R * n_around + 1
    faces = []
    j = np.arange(n_around)
    jn = (j + 1) % n_around
    for k in range(R - 1):
        a, b = k * n_around + j, k * n_around + jn
        c, d = (k + 1) * n_around + j, (k + 1) * n_around + jn
        faces.append(np.stack([a, b, d], 1))
        faces.append(np.stack([a, d, c], 1))
    faces.append(np.stack([np.full(n_around, bot), jn, j], 1))
    last = (R - 1) * n_around
    faces.append(np.stack([np.full(n_around, top), last + j, last + jn], 1))
    f = np.concatenate(faces)
    # orient outward: flip faces whose normal points toward the axis
    t = xyz[f]
    cn = np.cross(t[:, 1] - t[:, 0], t[:, 2] - t[:, 0])
    cen = t.mean(axis=1)
    s = np.clip(((cen - p0) @ w) / length, 0.0, 1.0)
    radial = cen - (p0[None, :] + s[:, None] * axis[None, :])
    flip = (cn * radial).sum(1) < 0
    f[flip] = f[flip][:, [0, 2, 1]]
    return Body(xyz=np.ascontiguousarray(xyz, np.float32), tris=np.ascontiguousarray(f, np.uint32),
                normals=np.ascontiguousarray(nrm, np.float32))


def merge_bodies(parts: list[Body]) -> Body:
    xyz, tris, nrm, off = [], [], [], 0
    for b in parts:
        xyz.append(b.xyz)
        tris.append(b.tris + off)
        nrm.append(b.normals)
        off += len(b.xyz)
    return Body(xyz=np.concatenate(xyz), tris=np.ascontiguousarray(np.concatenate(tris), np.uint32),
                normals=np.concatenate(nrm))


def three_capsules(center=(0.0, -0.55, 0.0)) -> Body:
    """Torso (r = 0.15 m) and two arms (r = 0.05 m): 19,392 triangles."""
    c = np.asarray(center, np.float64)
    torso = capsule(c + [0, -0.25, 0], c + [0, 0.25, 0], 0.15, 96, 60)
    arm_l = capsule(c + [-0.2, 0.2, 0], c + [-0.65, 0.2, 0], 0.05, 48, 42)
    arm_r = capsule(c + [0.2, 0.2, 0], c + [0.65, 0.2, 0], 0.05, 48, 42)
    return merge_bodies([torso, arm_l, arm_r])


def translated(body: Body, offset) -> np.ndarray:
    return (body.xyz.astype(np.float64) + np.asarray(offset, np.float64)[None, :]).astype(np.float32)


# --------------------------------------------------------------------------------------
# the benchmark workloads
# --------------------------------------------------------------------------------------
def config_physics(substeps: int = 2):
    """Physics of the synthetic workloads: k = 2000 / 1000 / 500 N/m, m = 1e-3 kg,
    g = -9.8, Verlet damping 0.99 per 1e-3 s frame, 5 mm thickness.  The frame is
    split into `substeps` steps (gamma = 0.99 ** (1 / substeps) per step, spring
    damping off): one explicit step per 1e-3 s frame is linearly unstable at these
    stiffnesses (omega_max * dt ~ 3.45 > 2)."""
    return dict(dt=1e-3 / substeps, mass=1e-3, gravity=(0.0, -9.8, 0.0), force_damping=0.0,
                spring_damping=0.0, verlet_damping=0.99 ** (1.0 / substeps), thickness=0.005, box_depth=0.01,
                list_k=(2000.0, 1000.0, 500.0))


def physics_params(substeps: int = 2, **overrides):
    """VisgParams of config_physics (three spring lists)."""
    from .params import make_params
    ph = config_physics(substeps)
    ph.update(overrides)
    return make_params(3, ph["dt"], ph["mass"], ph["gravity"], ph["force_damping"], ph["spring_damping"],
                       ph["verlet_damping"], ph["thickness"], ph["box_depth"], ph["list_k"])


def garment_over_capsules(seed: int = 0):
    """The garment-scale plain workload: a 112 x 112 sheet (1 m) with positions
    jittered by N(0, 1e-4 m), two corners pinned, over a torso and two arms
    (19,392 triangles) that translate along -y at 0.5 m/s (the LBVH is rebuilt every
    step).  Returns (cloth, body, motion) with motion(t) the body offset at time t."""
    cloth = grid_cloth(112, 1.0, 0.0, jitter=1e-4, seed=seed)
    body = three_capsules()
    return cloth, body, lambda t: np.array([0.0, -0.5 * t, 0.0])


def sheet_over_noisy_sphere(seed: int = 0):
    """The large plain workload: a 512 x 512 sheet (1 m), two corners pinned, over an
    icosphere of subdivision 7 (327,680 triangles, radius 0.3 m, vertices radially
    perturbed by U(+-2%)) centred 0.5 m below, oscillating along y on a 1 Hz sine of
    amplitude 0.1 m (the LBVH is rebuilt every step)."""
    cloth = grid_cloth(512, 1.0, 0.0)
    body = icosphere(7, 0.3, center=(0.0, -0.5, 0.0), noise=0.02, seed=seed)
    return cloth, body, lambda t: np.array([0.0, 0.1 * np.sin(2.0 * np.pi * t), 0.0])


def sheet_over_sphere(side: int = 64, subdiv: int = 4, radius: float = 0.3, seed: int = 0):
    """64x64 sheet (1 m) with two pinned corners above an icosphere 0.5 m below."""
    cloth = grid_cloth(side, 1.0, 0.0)
    body = icosphere(subdiv, radius, center=(0.0, -0.5, 0.0))
    return cloth, body


def garment_batch(n_garments: int = 256, seed: int = 0, side_range=(32, 256), subdiv_range=(3, 6),
                  radius_range=(0.2, 0.4), centre_depth: float = 0.5, cap: float | None = None,
                  pin_corners: bool = True):
    """Per garment: side ~ U{32..256}, a 1 m sheet with the three spring families and
    two pinned corners, facing an icosphere of subdivision ~ U{3..6} and radius
    ~ U[0.2, 0.4] m centred `centre_depth` metres below the sheet (the single-sheet
    workload's placement); the sheet falls onto it.  With `cap`, the sphere's top
    instead rises `cap` metres through the sheet (cap > 0 starts with a deep overlap
    that the first step projects out: violent, and unstable at these stiffnesses)."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(side_range[0], side_range[1] + 1, size=n_garments)
    subs = rng.integers(subdiv_range[0], subdiv_range[1] + 1, size=n_garments)
    radii = rng.uniform(radius_range[0], radius_range[1], size=n_garments)
    spheres = {}
    out = []
    for g in range(n_garments):
        cloth = grid_cloth(int(sides[g]), 1.0, 0.0, pin_top_corners=pin_corners)
        key = int(subs[g])
        if key not in spheres:
            spheres[key] = icosphere(key, 1.0)
        unit = spheres[key]
        r = float(radii[g])
        cy = -centre_depth if cap is None else cap - r
        body = Body(xyz=(unit.xyz.astype(np.float64) * r + np.array([0.0, cy, 0.0])).astype(np.float32),
                    tris=unit.tris, normals=unit.normals)
        out.append((cloth, body))
    return out
