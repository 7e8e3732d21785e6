"""ctypes mirror of the C structs in include/visg_sim.h (no library is loaded here)."""
from __future__ import annotations

import ctypes as C

VISG_MAX_LISTS = 4

STATUS = {
    0: "VISG_OK", -1: "VISG_ERR_INVALID_ARG", -2: "VISG_ERR_CUDA", -3: "VISG_ERR_OOM",
    -4: "VISG_ERR_NO_DEVICE", -5: "VISG_ERR_DIVERGED", -6: "VISG_ERR_TIMEOUT",
    -7: "VISG_ERR_STATE", -8: "VISG_ERR_UNSUPPORTED",
}


class VisgParams(C.Structure):
    _fields_ = [
        ("dt", C.c_float),
        ("mass", C.c_float),
        ("gravity", C.c_float * 3),
        ("force_damping", C.c_float),
        ("spring_damping", C.c_float),
        ("verlet_damping", C.c_float),
        ("thickness", C.c_float),
        ("box_depth", C.c_float),
        ("n_lists", C.c_int32),
        ("list_k", C.c_float * VISG_MAX_LISTS),
        ("collide", C.c_int32),
        ("check_every", C.c_int32),
        ("max_displacement", C.c_float),
        ("use_graph", C.c_int32),
        ("split_collision", C.c_int32),
        ("stage_neighbours", C.c_int32),
        ("collision_margin", C.c_int32),
        ("overlap_groups", C.c_int32),
    ]


def reference_params(n_lists: int = 2) -> VisgParams:
    """The reference's constants (src/verlet.cu:12-21,62; src/simulation.cu:132;
    src/bvh/primitive.cu:21): dt = 1/40, m = 0.3, g = (0, -0.00981, 0), force damping
    -0.02, spring kd -0.5, structure k = 100, bend k = 2, thickness 0.003, depth 0.01."""
    p = VisgParams()
    p.dt = 1.0 / 40.0
    p.mass = 0.3
    p.gravity[:] = (0.0, -0.00981, 0.0)
    p.force_damping = -0.02
    p.spring_damping = -0.5
    p.verlet_damping = 1.0
    p.thickness = 0.003
    p.box_depth = 0.01
    p.n_lists = n_lists
    p.list_k[:] = (100.0, 2.0, 2.0, 2.0)
    p.collide = 1
    p.check_every = 0
    p.max_displacement = 1.0
    p.use_graph = 1
    p.split_collision = 1
    p.stage_neighbours = 0
    p.collision_margin = 1
    p.overlap_groups = 0
    return p


def make_params(n_lists: int, dt: float, mass: float, gravity=(0.0, -9.8, 0.0), force_damping=0.0,
                spring_damping=0.0, verlet_damping=1.0, thickness=0.003, box_depth=0.01,
                list_k=(100.0, 2.0, 2.0, 2.0), collide=1, check_every=0, max_displacement=1.0,
                use_graph=1, split_collision=1, stage_neighbours=0,
                collision_margin=1, overlap_groups=0) -> VisgParams:
    p = VisgParams()
    p.dt, p.mass = dt, mass
    p.gravity[:] = tuple(gravity)
    p.force_damping, p.spring_damping, p.verlet_damping = force_damping, spring_damping, verlet_damping
    p.thickness, p.box_depth = thickness, box_depth
    p.n_lists = n_lists
    k = list(list_k) + [0.0] * (VISG_MAX_LISTS - len(list_k))
    p.list_k[:] = tuple(k[:VISG_MAX_LISTS])
    p.collide, p.check_every, p.max_displacement, p.use_graph = collide, check_every, max_displacement, use_graph
    p.split_collision = split_collision
    p.stage_neighbours = stage_neighbours
    p.collision_margin = collision_margin
    p.overlap_groups = overlap_groups
    return p
