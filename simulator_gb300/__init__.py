"""GB300-native VISGSim cloth step: Python mirror of the reference's Simulator.

The compute path is the CUDA library simulator_gb300/_lib/libvisgsim.so
(include/visg_sim.h); this module only marshals numpy arrays through its C ABI.
There is no CPU fallback: constructing a Simulator without the built library or
without a GPU raises.

Reference interface (src/simulator.h:9-59) -> this module:
    Simulator(Mesh& cloth, Mesh& body)   -> Simulator(cloth, body, params)
    simulate(Mesh*)                      -> Simulator.simulate(nsteps=1)
    update_vertex(glm::vec3, idx)        -> Simulator.update_vertex(new_value, idx)
    cuda_update_vbo(Mesh*)               -> Simulator.positions() (headless)
    (new) body motion                    -> Simulator.update_body(xyz, normals)
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .params import STATUS, VisgParams, make_params, reference_params  # noqa: F401
from . import scenes  # noqa: F401

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libvisgsim.so")

_fp = C.POINTER(C.c_float)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_i64p = C.POINTER(C.c_int64)
_vp = C.c_void_p

_lib = None


class VisgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def lib():
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"CUDA library not built: {LIB_PATH}; run __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    sig = {
        "visg_default_params": (None, [C.POINTER(VisgParams)]),
        "visg_version": (C.c_char_p, []),
        "visg_selftest_bounded_waits": (C.c_int, [_i32p]),
        "visg_selftest_exact_math": (C.c_int, [C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
        "visg_batch_time_kernels": (C.c_int, [_vp, C.c_int32, _fp, _fp]),
        "visg_last_error": (C.c_char_p, []),
        "visg_create": (C.c_int, [C.POINTER(VisgParams), _fp, C.c_int32, C.POINTER(_u32p), C.POINTER(_vp),
                                  C.POINTER(_fp), _fp, _fp, C.c_int32, _u32p, C.c_int32, C.POINTER(_vp)]),
        "visg_destroy": (C.c_int, [_vp]),
        "visg_set_stream": (C.c_int, [_vp, _vp]),
        "visg_step": (C.c_int, [_vp, C.c_int32]),
        "visg_update_body": (C.c_int, [_vp, _fp, _fp]),
        "visg_update_body_device": (C.c_int, [_vp, _vp, _vp]),
        "visg_set_vertex": (C.c_int, [_vp, C.c_uint32, _fp]),
        "visg_set_pinned": (C.c_int, [_vp, _u32p, C.c_int32]),
        "visg_set_vertices": (C.c_int, [_vp, _u32p, _fp, C.c_int32]),
        "visg_batch_set_vertices": (C.c_int, [_vp, _u32p, _fp, C.c_int32]),
        "visg_get_positions": (C.c_int, [_vp, _vp, C.c_int32]),
        "visg_get_state": (C.c_int, [_vp, _fp, _fp, _fp]),
        "visg_set_state": (C.c_int, [_vp, _fp, _fp, _fp]),
        "visg_sync": (C.c_int, [_vp]),
        "visg_count_contacts": (C.c_int, [_vp, _i64p]),
        "visg_batch_count_contacts": (C.c_int, [_vp, _i64p]),
        "visg_get_info": (C.c_int, [_vp, _i32p, _i32p, _i32p, _i32p]),
        "visg_export_lbvh": (C.c_int, [_vp, _u32p, _fp, _u32p, _i32p, _i32p, _i32p, _i32p, _i32p, _fp, _fp, _fp]),
        "visg_query_points": (C.c_int, [_vp, _fp, C.c_int32, _i32p, _i32p, _fp, _fp]),
        "visg_forward": (C.c_int, [_vp, C.c_int32, C.c_int32]),
        "visg_backward": (C.c_int, [_vp, _fp, _fp, _fp, _fp]),
        "visg_forward_contacts": (C.c_int, [_vp, C.POINTER(C.c_int64), C.c_int32]),
        "visg_batch_create": (C.c_int, [C.POINTER(VisgParams), C.POINTER(_vp)]),
        "visg_batch_add": (C.c_int, [_vp, _fp, C.c_int32, C.POINTER(_u32p), C.POINTER(_vp), C.POINTER(_fp),
                                     _u32p, C.c_int32, _fp, _fp, C.c_int32, _u32p, C.c_int32, _i32p]),
        "visg_batch_finalize": (C.c_int, [_vp]),
        "visg_batch_set_stream": (C.c_int, [_vp, _vp]),
        "visg_batch_step": (C.c_int, [_vp, C.c_int32]),
        "visg_batch_get_positions": (C.c_int, [_vp, C.c_int32, _vp, C.c_int32]),
        "visg_batch_set_vertex": (C.c_int, [_vp, C.c_int32, C.c_uint32, _fp]),
        "visg_batch_update_body": (C.c_int, [_vp, C.c_int32, _fp, _fp]),
        "visg_batch_autotune": (C.c_int, [_vp, _i32p, _i32p]),
        "visg_autotune": (C.c_int, [_vp, _i32p, _i32p]),
        "visg_batch_set_reserve": (C.c_int, [_vp, C.c_int32]),
        "visg_batch_get_reserve": (C.c_int, [_vp, _i32p]),
        "visg_launch_info": (C.c_int, [_vp, _i32p, _i32p, _i32p, _i32p, _i32p]),
        "visg_batch_set_launch": (C.c_int, [_vp, C.c_int32, C.c_int32]),
        "visg_batch_launch_info": (C.c_int, [_vp, _i32p, _i32p, _i32p, _i32p, _i32p]),
        "visg_batch_read_positions_async": (C.c_int, [_vp, _vp]),
        "visg_batch_get_state": (C.c_int, [_vp, C.c_int32, _fp, _fp, _fp]),
        "visg_batch_set_state": (C.c_int, [_vp, C.c_int32, _fp, _fp, _fp]),
        "visg_batch_wait_positions": (C.c_int, [_vp]),
        "visg_read_positions_async": (C.c_int, [_vp, _vp]),
        "visg_set_faces": (C.c_int, [_vp, _u32p, C.c_int32]),
        "visg_obj_load": (C.c_int, [C.c_char_p, C.POINTER(_vp), _i32p, _i32p]),
        "visg_obj_get": (C.c_int, [_vp, _fp, _fp, _u32p]),
        "visg_obj_free": (None, [_vp]),
        "visg_obj_groups": (C.c_int, [_vp, _i32p, _i32p]),
        "visg_springs_from_mesh_sewn": (C.c_int, [_fp, C.c_int32, _u32p, C.c_int32, _i32p, C.c_int32, _u32p,
                                                  _vp, _i32p, _u32p, _vp, _i32p]),
        "visg_mesh_scale": (C.c_int, [_fp, C.c_int32, C.c_float]),
        "visg_mesh_translate": (C.c_int, [_fp, C.c_int32, C.c_float, C.c_float, C.c_float]),
        "visg_mesh_rotate": (C.c_int, [_fp, C.c_int32, C.c_float, C.c_int32]),
        "visg_render": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int32, C.c_int32]),
        "visg_render_shaded": (C.c_int, [_vp, _vp, _vp, _vp, _fp, C.c_int32, C.c_int32]),
        "visg_batch_render_shaded": (C.c_int, [_vp, _vp, _vp, _vp, _fp, C.c_int32, C.c_int32]),
        "visg_batch_set_faces": (C.c_int, [_vp, C.c_int32, _u32p, C.c_int32]),
        "visg_batch_render": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int32, C.c_int32]),
        "visg_wait_positions": (C.c_int, [_vp]),
        "visg_batch_info": (C.c_int, [_vp, _i32p, _i64p, _i64p, _i64p]),
        "visg_batch_sync": (C.c_int, [_vp]),
        "visg_batch_destroy": (C.c_int, [_vp]),
        "visg_springs_from_mesh": (C.c_int, [_fp, C.c_int32, _u32p, C.c_int32, _u32p, _vp, _i32p, _u32p, _vp, _i32p]),
        "visg_lbvh_build_noalloc": (C.c_int, [_vp, _vp, C.c_int32, _vp, C.c_int32, C.c_float, C.c_float, _vp, _vp,
                                              _vp, _vp, _vp, _vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(code: int):
    if code != 0:
        raise VisgError(code, (lib().visg_last_error() or b"").decode())


def _p(a, t=_fp):
    return None if a is None else a.ctypes.data_as(t)


def _f32(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


def _lists_ctypes(lists, keep):
    L = len(lists)
    rows = (_u32p * L)()
    ents = (_vp * L)()
    ks = (_fp * L)()
    for i, sl in enumerate(lists):
        r = np.ascontiguousarray(sl.row, np.uint32)
        e = np.ascontiguousarray(sl.ent)
        keep += [r, e]
        rows[i] = r.ctypes.data_as(_u32p)
        ents[i] = e.ctypes.data
        if getattr(sl, "k", None) is not None:
            k = np.ascontiguousarray(sl.k, np.float32)
            keep.append(k)
            ks[i] = k.ctypes.data_as(_fp)
    return rows, ents, ks


class Simulator:
    """One garment over one body (the reference's Simulator, src/simulation.cu)."""

    def __init__(self, cloth_xyz, lists, body_xyz=None, body_tris=None, body_normals=None,
                 params: VisgParams | None = None, pinned=None):
        L = lib()
        self.params = params if params is not None else reference_params(len(lists))
        keep = []
        xyz = _f32(cloth_xyz)
        self.n = len(xyz)
        rows, ents, ks = _lists_ctypes(lists, keep)
        bx = _f32(body_xyz) if body_xyz is not None else np.zeros((0, 3), np.float32)
        bt = np.ascontiguousarray(body_tris, np.uint32) if body_tris is not None else np.zeros((0, 3), np.uint32)
        bn = _f32(body_normals)
        self.n_tris = len(bt)
        self.n_body_vertices = len(bx)
        self.has_normals = bn is not None
        self.n_entries = [int(sl.row[-1]) for sl in lists]
        h = _vp()
        _check(L.visg_create(C.byref(self.params), _p(xyz), self.n, rows, ents, ks, _p(bx), _p(bn), len(bx),
                             _p(bt, _u32p), len(bt), C.byref(h)))
        self.h = h
        if pinned is not None and len(pinned):
            self.set_pinned(pinned)

    # ---- lifetime
    def close(self):
        if getattr(self, "h", None):
            lib().visg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- reference surface
    def simulate(self, nsteps: int = 1):
        _check(lib().visg_step(self.h, nsteps))

    def update_vertex(self, new_value, idx: int):
        v = _f32(new_value).reshape(3)
        _check(lib().visg_set_vertex(self.h, idx, _p(v)))

    def update_vertices(self, idx, xyz):
        a = np.ascontiguousarray(idx, np.uint32)
        v = _f32(xyz).reshape(-1, 3)
        _check(lib().visg_set_vertices(self.h, _p(a, _u32p), _p(v), len(a)))

    def update_body(self, xyz, normals=None):
        _check(lib().visg_update_body(self.h, _p(_f32(xyz)), _p(_f32(normals))))

    def update_body_device(self, xyz_ptr: int, normals_ptr: int | None = None):
        _check(lib().visg_update_body_device(self.h, xyz_ptr, normals_ptr))

    def set_pinned(self, idx):
        a = np.ascontiguousarray(idx, np.uint32)
        _check(lib().visg_set_pinned(self.h, _p(a, _u32p), len(a)))

    def set_stream(self, stream_handle: int | None):
        _check(lib().visg_set_stream(self.h, stream_handle))

    def positions(self, out=None):
        out = np.empty((self.n, 3), np.float32) if out is None else out
        _check(lib().visg_get_positions(self.h, out.ctypes.data, 0))
        return out

    def positions_device(self, dev_ptr: int):
        _check(lib().visg_get_positions(self.h, dev_ptr, 1))

    def set_faces(self, faces):
        """The cloth's triangles ((F, 3) vertex indices), for render()."""
        f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
        self.n_faces = len(f)
        _check(lib().visg_set_faces(self.h, _p(f, _u32p), len(f)))

    def render(self, normals_of_previous: bool = True):
        """The output stage of cuda_update_vbo: (pos4 (n, 4), vertex normals (n, 3),
        face normals (F, 3)) as host arrays."""
        pos4 = np.empty((self.n, 4), np.float32)
        vn = np.empty((self.n, 3), np.float32)
        fn = np.empty((max(getattr(self, "n_faces", 0), 1), 3), np.float32)
        _check(lib().visg_render(self.h, pos4.ctypes.data, vn.ctypes.data, fn.ctypes.data, 0,
                                 1 if normals_of_previous else 0))
        return pos4, vn, fn[:getattr(self, "n_faces", 0)]

    def render_shaded(self, object_rgb=(1.0, 1.0, 1.0), normals_of_previous: bool = True):
        """(pos4, vertex normals, SH-shaded colours (n, 3)) as host arrays."""
        pos4 = np.empty((self.n, 4), np.float32)
        vn = np.empty((self.n, 3), np.float32)
        col = np.empty((self.n, 3), np.float32)
        rgb = np.ascontiguousarray(object_rgb, np.float32)
        _check(lib().visg_render_shaded(self.h, pos4.ctypes.data, vn.ctypes.data, col.ctypes.data, _p(rgb), 0,
                                        1 if normals_of_previous else 0))
        return pos4, vn, col

    def read_positions_async(self, out):
        """Enqueue the read of all positions into `out` ((n, 3) float32, ideally
        page-locked) behind the steps issued so far; returns at once."""
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == 3 * self.n
        _check(lib().visg_read_positions_async(self.h, out.ctypes.data))

    def wait_positions(self):
        """Wait for the oldest read in flight."""
        _check(lib().visg_wait_positions(self.h))

    def state(self):
        x, xo, n = (np.empty((self.n, 3), np.float32) for _ in range(3))
        _check(lib().visg_get_state(self.h, _p(x), _p(xo), _p(n)))
        return x, xo, n

    def set_state(self, x=None, xo=None, n=None):
        _check(lib().visg_set_state(self.h, _p(_f32(x)), _p(_f32(xo)), _p(_f32(n))))

    def sync(self):
        _check(lib().visg_sync(self.h))

    def count_contacts(self) -> int:
        n = C.c_int64()
        _check(lib().visg_count_contacts(self.h, C.byref(n)))
        return n.value

    def info(self):
        a, b, c, d = (C.c_int32() for _ in range(4))
        _check(lib().visg_get_info(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return dict(n_vertices=a.value, n_entries=b.value, n_tris=c.value, n_leaves=d.value)

    def autotune(self):
        """Time the step kernel's launch shapes and variants on this simulator's data
        and keep the fastest (the state is unchanged); returns (block, ctas_per_sm)."""
        b, c = C.c_int32(), C.c_int32()
        _check(lib().visg_autotune(self.h, C.byref(b), C.byref(c)))
        return b.value, c.value

    def launch_info(self) -> dict:
        v = [C.c_int32() for _ in range(5)]
        _check(lib().visg_launch_info(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("block", "ctas_per_sm", "split_collision", "stage_neighbours", "kernels_per_step"),
                        (x.value for x in v)))

    def export_lbvh(self) -> dict:
        T = self.n_tris
        Tp = self.info()["n_leaves"]
        ni = max(Tp - 1, 0)
        o = dict(tri_codes=np.zeros(T, np.uint32), tri_boxes=np.zeros((T, 6), np.float32),
                 sorted_codes=np.zeros(Tp, np.uint32), sorted_tris=np.zeros(Tp, np.int32),
                 child_a=np.zeros(ni, np.int32), child_b=np.zeros(ni, np.int32),
                 parent_internal=np.zeros(ni, np.int32), parent_leaf=np.zeros(Tp, np.int32),
                 internal_boxes=np.zeros((ni, 6), np.float32), leaf_boxes=np.zeros((Tp, 6), np.float32),
                 root_box=np.zeros(6, np.float32))
        _check(lib().visg_export_lbvh(self.h, _p(o["tri_codes"], _u32p), _p(o["tri_boxes"]),
                                      _p(o["sorted_codes"], _u32p), _p(o["sorted_tris"], _i32p),
                                      _p(o["child_a"], _i32p), _p(o["child_b"], _i32p),
                                      _p(o["parent_internal"], _i32p), _p(o["parent_leaf"], _i32p),
                                      _p(o["internal_boxes"]), _p(o["leaf_boxes"]), _p(o["root_box"])))
        o["n_leaves"] = Tp
        return o

    def query(self, pts):
        pts = _f32(pts)
        n = len(pts)
        leaf, inside = np.zeros(n, np.int32), np.zeros(n, np.int32)
        dist, nrm = np.zeros(n, np.float32), np.zeros((n, 3), np.float32)
        _check(lib().visg_query_points(self.h, _p(pts), n, _p(leaf, _i32p), _p(inside, _i32p), _p(dist), _p(nrm)))
        return leaf, inside, dist, nrm

    # ---- differentiation
    def forward(self, nsteps: int, checkpoint_every: int = 50):
        _check(lib().visg_forward(self.h, nsteps, checkpoint_every))
        self._fwd_steps = nsteps

    def forward_contacts(self):
        """Vertices projected in each step of the last forward() (the frozen active set)."""
        c = np.zeros(getattr(self, "_fwd_steps", 0), np.int64)
        _check(lib().visg_forward_contacts(self.h, c.ctypes.data_as(C.POINTER(C.c_int64)), len(c)))
        return c

    def backward(self, dL_dx, dL_dxo=None):
        dk = np.zeros(sum(self.n_entries), np.float32)
        ds = np.zeros(3, np.float32)
        _check(lib().visg_backward(self.h, _p(_f32(dL_dx)), _p(_f32(dL_dxo)), _p(dk), _p(ds)))
        return dk, ds


class BatchSimulator:
    """Many garments, each with its own body; every kernel launch covers many garments
    (by default two garment groups, each its own overlapping chain of kernels)."""

    def __init__(self, params: VisgParams):
        L = lib()
        self.params = params
        h = _vp()
        _check(L.visg_batch_create(C.byref(params), C.byref(h)))
        self.h = h
        self.sizes = []
        self.finalized = False

    def add(self, cloth_xyz, lists, body_xyz=None, body_tris=None, body_normals=None, pinned=None) -> int:
        keep = []
        xyz = _f32(cloth_xyz)
        rows, ents, ks = _lists_ctypes(lists, keep)
        bx = _f32(body_xyz) if body_xyz is not None else np.zeros((0, 3), np.float32)
        bt = np.ascontiguousarray(body_tris, np.uint32) if body_tris is not None else np.zeros((0, 3), np.uint32)
        bn = _f32(body_normals)
        pins = np.ascontiguousarray(pinned if pinned is not None else np.zeros(0), np.uint32)
        g = C.c_int32()
        _check(lib().visg_batch_add(self.h, _p(xyz), len(xyz), rows, ents, ks, _p(pins, _u32p), len(pins), _p(bx),
                                    _p(bn), len(bx), _p(bt, _u32p), len(bt), C.byref(g)))
        self.sizes.append(len(xyz))
        return g.value

    def finalize(self):
        _check(lib().visg_batch_finalize(self.h))
        self.finalized = True
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)

    def step(self, nsteps: int = 1):
        _check(lib().visg_batch_step(self.h, nsteps))

    def set_stream(self, stream_handle: int | None):
        _check(lib().visg_batch_set_stream(self.h, stream_handle))

    def positions(self, garment: int = -1, out=None):
        n = int(self.offsets[-1]) if garment < 0 else self.sizes[garment]
        out = np.empty((n, 3), np.float32) if out is None else out
        _check(lib().visg_batch_get_positions(self.h, garment, out.ctypes.data, 0))
        return out

    def positions_device(self, dev_ptr: int, garment: int = -1):
        _check(lib().visg_batch_get_positions(self.h, garment, dev_ptr, 1))

    def set_faces(self, garment: int, faces):
        f = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
        if not hasattr(self, "face_counts"):
            self.face_counts = {}
        self.face_counts[garment] = len(f)
        _check(lib().visg_batch_set_faces(self.h, garment, _p(f, _u32p), len(f)))

    def render(self, normals_of_previous: bool = True):
        n = int(self.offsets[-1])
        nf = sum(getattr(self, "face_counts", {}).values())
        pos4 = np.empty((n, 4), np.float32)
        vn = np.empty((n, 3), np.float32)
        fn = np.empty((max(nf, 1), 3), np.float32)
        _check(lib().visg_batch_render(self.h, pos4.ctypes.data, vn.ctypes.data, fn.ctypes.data, 0,
                                       1 if normals_of_previous else 0))
        return pos4, vn, fn[:nf]

    def read_positions_async(self, out):
        """Enqueue the read of every garment's positions (concatenated) into `out`
        ((n, 3) float32, ideally page-locked) behind the steps issued so far."""
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == 3 * int(self.offsets[-1])
        _check(lib().visg_batch_read_positions_async(self.h, out.ctypes.data))

    def wait_positions(self):
        """Wait for the oldest read in flight."""
        _check(lib().visg_batch_wait_positions(self.h))

    def update_vertex(self, garment: int, new_value, idx: int):
        v = _f32(new_value).reshape(3)
        _check(lib().visg_batch_set_vertex(self.h, garment, idx, _p(v)))

    def update_vertices(self, idx, xyz):
        """idx: global vertex indices (garments concatenated in id order)."""
        a = np.ascontiguousarray(idx, np.uint32)
        v = _f32(xyz).reshape(-1, 3)
        _check(lib().visg_batch_set_vertices(self.h, _p(a, _u32p), _p(v), len(a)))

    def update_body(self, garment: int, xyz, normals=None):
        _check(lib().visg_batch_update_body(self.h, garment, _p(_f32(xyz)), _p(_f32(normals))))

    def time_kernels(self, nsteps: int = 10):
        """Step nsteps times as one chain with CUDA events around each kernel launch:
        (ms per step-kernel launch, ms per collision pass), device time averages."""
        a, c = C.c_float(), C.c_float()
        _check(lib().visg_batch_time_kernels(self.h, nsteps, C.byref(a), C.byref(c)))
        return a.value, c.value

    def autotune(self):
        b, c = C.c_int32(), C.c_int32()
        _check(lib().visg_batch_autotune(self.h, C.byref(b), C.byref(c)))
        return b.value, c.value

    def state(self, garment: int = -1):
        n = int(self.offsets[-1]) if garment < 0 else self.sizes[garment]
        x, xo, nr = (np.empty((n, 3), np.float32) for _ in range(3))
        _check(lib().visg_batch_get_state(self.h, garment, _p(x), _p(xo), _p(nr)))
        return x, xo, nr

    def set_state(self, garment: int = -1, x=None, xo=None, n=None):
        _check(lib().visg_batch_set_state(self.h, garment, _p(_f32(x)), _p(_f32(xo)), _p(_f32(n))))

    def launch_info(self) -> dict:
        v = [C.c_int32() for _ in range(5)]
        _check(lib().visg_batch_launch_info(self.h, *[C.byref(x) for x in v]))
        d = dict(zip(("block", "ctas_per_sm", "split_collision", "stage_neighbours", "kernels_per_step"),
                     (x.value for x in v)))
        r = C.c_int32()
        _check(lib().visg_batch_get_reserve(self.h, C.byref(r)))
        d["sms_left_to_collision"] = r.value
        return d

    def set_launch(self, block: int, ctas_per_sm: int):
        _check(lib().visg_batch_set_launch(self.h, block, ctas_per_sm))

    def set_reserve(self, sms: int):
        """SMs the step kernel leaves to the other garment group's collision pass."""
        _check(lib().visg_batch_set_reserve(self.h, sms))

    def info(self):
        g = C.c_int32()
        v, e, t = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().visg_batch_info(self.h, C.byref(g), C.byref(v), C.byref(e), C.byref(t)))
        return dict(n_garments=g.value, n_vertices=v.value, n_entries=e.value, n_tris=t.value)

    def sync(self):
        _check(lib().visg_batch_sync(self.h))

    def count_contacts(self) -> int:
        n = C.c_int64()
        _check(lib().visg_batch_count_contacts(self.h, C.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "h", None):
            lib().visg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def selftest_bounded_waits() -> int:
    """Run the device-side failure-detection self-test (visg_selftest_bounded_waits):
    a staging-ring wait, a radix look-back wait and an LBVH grid-barrier wait that
    nothing completes must all give up and report it.  Returns the bits of the waits
    that gave up (7 = all three)."""
    bits = C.c_int32()
    _check(lib().visg_selftest_bounded_waits(C.byref(bits)))
    return bits.value


def selftest_exact_math() -> tuple[int, int]:
    """Run visg_selftest_exact_math: the step's packed square root and reciprocal on
    every float of their range against the CUDA intrinsics; (checked, mismatches)."""
    n, bad = C.c_uint64(0), C.c_uint64(0)
    _check(lib().visg_selftest_exact_math(C.byref(n), C.byref(bad)))
    return int(n.value), int(bad.value)


def springs_from_mesh(xyz, tris):
    """Reference spring topology from a triangle mesh (structure list, bend list)."""
    from .scenes import SPRING_DTYPE, SpringList
    xyz = _f32(xyz)
    tris = np.ascontiguousarray(tris, np.uint32)
    nv, nt = len(xyz), len(tris)
    n0, n1 = C.c_int32(), C.c_int32()
    _check(lib().visg_springs_from_mesh(_p(xyz), nv, _p(tris, _u32p), nt, None, None, C.byref(n0), None, None,
                                        C.byref(n1)))
    r0, r1 = np.zeros(nv + 1, np.uint32), np.zeros(nv + 1, np.uint32)
    e0, e1 = np.zeros(n0.value, SPRING_DTYPE), np.zeros(n1.value, SPRING_DTYPE)
    _check(lib().visg_springs_from_mesh(_p(xyz), nv, _p(tris, _u32p), nt, _p(r0, _u32p), e0.ctypes.data,
                                        C.byref(n0), _p(r1, _u32p), e1.ctypes.data, C.byref(n1)))
    return [SpringList(r0, e0), SpringList(r1, e1)]


def load_obj(path: str):
    """A Wavefront OBJ read as the reference's ObjLoader + Mesh::unified do:
    (xyz (V, 3) float32, per-vertex normals (V, 3), triangles (F, 3) uint32)."""
    h = _vp()
    nv, nf = C.c_int32(), C.c_int32()
    _check(lib().visg_obj_load(str(path).encode(), C.byref(h), C.byref(nv), C.byref(nf)))
    try:
        xyz = np.empty((nv.value, 3), np.float32)
        nrm = np.empty((nv.value, 3), np.float32)
        faces = np.empty((nf.value, 3), np.uint32)
        _check(lib().visg_obj_get(h, _p(xyz), _p(nrm), _p(faces, _u32p)))
    finally:
        lib().visg_obj_free(h)
    return xyz, nrm, faces


def mesh_scale(xyz, s: float):
    """Mesh::scale: (v - mean) * s, in place on a float32 (n, 3) array."""
    _check(lib().visg_mesh_scale(_p(xyz), len(xyz), s))
    return xyz


def mesh_translate(xyz, dx: float, dy: float, dz: float):
    _check(lib().visg_mesh_translate(_p(xyz), len(xyz), dx, dy, dz))
    return xyz


def mesh_rotate(xyz, angle_degrees: float, axis: int):
    """Mesh::rotation about the vertex mean; axis 0 = x, 1 = y, 2 = z."""
    _check(lib().visg_mesh_rotate(_p(xyz), len(xyz), angle_degrees, axis))
    return xyz


def write_obj(path: str, xyz, faces=None):
    """Positions (and triangles, 0-based) as a Wavefront OBJ ("v" and "f a b c")."""
    with open(path, "w") as f:
        for p in np.asarray(xyz, np.float32):
            f.write(f"v {p[0]:.9g} {p[1]:.9g} {p[2]:.9g}\n")
        if faces is not None:
            for t in np.asarray(faces, np.int64):
                f.write(f"f {t[0] + 1} {t[1] + 1} {t[2] + 1}\n")


def obj_groups(path: str):
    """Vertex group sizes of a multi-piece garment OBJ ("# object" / "# N vertices")."""
    h = _vp()
    nv, nf, ng = C.c_int32(), C.c_int32(), C.c_int32()
    _check(lib().visg_obj_load(str(path).encode(), C.byref(h), C.byref(nv), C.byref(nf)))
    try:
        _check(lib().visg_obj_groups(h, None, C.byref(ng)))
        g = np.zeros(ng.value, np.int32)
        _check(lib().visg_obj_groups(h, _p(g, _i32p), C.byref(ng)))
    finally:
        lib().visg_obj_free(h)
    return g


def springs_from_mesh_sewn(xyz, tris, group_sizes):
    """springs_from_mesh plus the seams of a multi-piece garment (the reference's
    SINGLE_LAYER_BOUNDARY): group_sizes = piece, boundary, piece, boundary, ..."""
    from .scenes import SPRING_DTYPE, SpringList
    xyz = _f32(xyz)
    tris = np.ascontiguousarray(tris, np.uint32)
    g = np.ascontiguousarray(group_sizes, np.int32)
    nv, nt = len(xyz), len(tris)
    n0, n1 = C.c_int32(), C.c_int32()
    _check(lib().visg_springs_from_mesh_sewn(_p(xyz), nv, _p(tris, _u32p), nt, _p(g, _i32p), len(g), None, None,
                                             C.byref(n0), None, None, C.byref(n1)))
    r0, r1 = np.zeros(nv + 1, np.uint32), np.zeros(nv + 1, np.uint32)
    e0, e1 = np.zeros(n0.value, SPRING_DTYPE), np.zeros(n1.value, SPRING_DTYPE)
    _check(lib().visg_springs_from_mesh_sewn(_p(xyz), nv, _p(tris, _u32p), nt, _p(g, _i32p), len(g),
                                             _p(r0, _u32p), e0.ctypes.data, C.byref(n0), _p(r1, _u32p),
                                             e1.ctypes.data, C.byref(n1)))
    return [SpringList(r0, e0), SpringList(r1, e1)]
