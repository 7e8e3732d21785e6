"""ctypes wrapper of the CPU oracle (oracle/visg_oracle.cpp).

Test infrastructure: used by tests/, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py as the checker, never by the library itself.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from simulator_gb300.params import VisgParams

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libvisg_oracle.so")
_lib = None

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"oracle library not built: {LIB_PATH} (run __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        L.orc_num_threads.argtypes = [C.c_int]
        L.orc_num_threads.restype = C.c_int
        L.orc_sim_create.restype = C.c_void_p
        L.orc_sim_create.argtypes = [C.c_int, C.POINTER(VisgParams), _fp, C.c_int, C.POINTER(_u32p),
                                     C.POINTER(C.c_void_p), C.POINTER(_fp), _fp, _fp, C.c_int, _u32p, C.c_int]
        L.orc_sim_destroy.argtypes = [C.c_void_p]
        L.orc_sim_step.argtypes = [C.c_void_p, C.c_int]
        L.orc_sim_update_body.argtypes = [C.c_void_p, _fp, _fp]
        L.orc_sim_set_vertex.argtypes = [C.c_void_p, C.c_int, _fp]
        L.orc_sim_set_pinned.argtypes = [C.c_void_p, _u32p, C.c_int]
        L.orc_sim_get_state.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.orc_sim_set_state.argtypes = [C.c_void_p, _fp, _fp, _fp]
        L.orc_sim_n_leaves.argtypes = [C.c_void_p]
        L.orc_sim_n_leaves.restype = C.c_int
        L.orc_sim_contact_hash.argtypes = [C.c_void_p]
        L.orc_sim_contact_hash.restype = C.c_uint64
        L.orc_sim_record_contacts.argtypes = [C.c_void_p, C.c_int]
        L.orc_sim_record_contacts.restype = C.c_void_p
        L.orc_sim_step_forced.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.orc_sim_step_forced.restype = C.c_int
        L.orc_contacts_free.argtypes = [C.c_void_p]
        L.orc_sim_export_lbvh.argtypes = [C.c_void_p, _u32p, _fp, _u32p, _i32p, _i32p, _i32p, _i32p, _i32p,
                                          _fp, _fp, _fp]
        L.orc_sim_query.argtypes = [C.c_void_p, _fp, C.c_int, _i32p, _i32p, _dp, _dp]
        L.orc_sim_forward.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
        L.orc_sim_forward.restype = C.c_int
        L.orc_sim_backward.argtypes = [C.c_void_p, C.c_void_p, _dp, _dp, _dp, _dp]
        L.orc_springs_from_mesh.argtypes = [_fp, C.c_int, _u32p, C.c_int, _u32p, C.c_void_p, _i32p,
                                            _u32p, C.c_void_p, _i32p]
        L.orc_render.argtypes = [_fp, _fp, C.c_int, _u32p, C.c_int, _fp, _fp, _fp]
        L.orc_sh_shade.argtypes = [_fp, C.c_int, _fp, _fp]
        _lib = L
    return _lib


def ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)


def num_threads(n: int = 0) -> int:
    return lib().orc_num_threads(n)


class ContactRecord:
    """A contact history recorded by OracleSim.record_contacts (freed on deletion)."""

    def __init__(self, h, nsteps):
        self.h, self.nsteps = h, nsteps

    def __del__(self):
        try:
            if self.h:
                lib().orc_contacts_free(self.h)
                self.h = None
        except Exception:
            pass


class OracleSim:
    """CPU restatement of one garment + body (prec = 4: reference float arithmetic,
    prec = 8: FP64 oracle)."""

    def __init__(self, params: VisgParams, xyz, lists, body_xyz=None, body_tris=None, body_normals=None,
                 prec: int = 4, pinned=None):
        self._keep = []
        xyz = np.ascontiguousarray(xyz, np.float32)
        self.n = len(xyz)
        L = len(lists)
        assert params.n_lists == L
        rows = (_u32p * L)()
        ents = (C.c_void_p * L)()
        ks = (_fp * L)()
        for i, sl in enumerate(lists):
            r = np.ascontiguousarray(sl.row, np.uint32)
            e = np.ascontiguousarray(sl.ent)
            self._keep += [r, e]
            rows[i] = r.ctypes.data_as(_u32p)
            ents[i] = e.ctypes.data
            if sl.k is not None:
                k = np.ascontiguousarray(sl.k, np.float32)
                self._keep.append(k)
                ks[i] = k.ctypes.data_as(_fp)
        self.n_entries = [int(sl.row[-1]) for sl in lists]
        if body_xyz is None:
            bx = np.zeros((0, 3), np.float32)
            bt = np.zeros((0, 3), np.uint32)
        else:
            bx = np.ascontiguousarray(body_xyz, np.float32)
            bt = np.ascontiguousarray(body_tris, np.uint32)
        bn = None if body_normals is None else np.ascontiguousarray(body_normals, np.float32)
        self.n_tris = len(bt)
        self.params = params
        self.h = lib().orc_sim_create(prec, C.byref(params), ptr(xyz, _fp), self.n, rows, ents, ks,
                                      ptr(bx, _fp), ptr(bn, _fp), len(bx), ptr(bt, _u32p), len(bt))
        if pinned is not None and len(pinned):
            self.set_pinned(pinned)

    def close(self):
        if getattr(self, "h", None):
            lib().orc_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n: int = 1):
        lib().orc_sim_step(self.h, n)

    def record_contacts(self, nsteps: int) -> "ContactRecord":
        """Step nsteps times, keeping the leaf every vertex was projected onto in every
        step (the contact history)."""
        return ContactRecord(lib().orc_sim_record_contacts(self.h, nsteps), nsteps)

    def step_forced(self, record: "ContactRecord", first: int = 0, n: int | None = None):
        """Replay steps [first, first + n) of a contact history instead of deciding
        contacts: the projections of the record, by the branch's own formula."""
        n = record.nsteps - first if n is None else n
        if lib().orc_sim_step_forced(self.h, record.h, first, n) != 0:
            raise RuntimeError("contact record does not fit this simulator or range")

    def contact_hash(self) -> int:
        """Running hash of every step's contact set (projected vertices and their
        normals) since creation: equal hashes = equal contact sets in every step."""
        return int(lib().orc_sim_contact_hash(self.h))

    def update_body(self, xyz, normals=None):
        xyz = np.ascontiguousarray(xyz, np.float32)
        nn = None if normals is None else np.ascontiguousarray(normals, np.float32)
        lib().orc_sim_update_body(self.h, ptr(xyz, _fp), ptr(nn, _fp))

    def set_vertex(self, idx: int, xyz):
        v = np.ascontiguousarray(xyz, np.float32)
        lib().orc_sim_set_vertex(self.h, idx, ptr(v, _fp))

    def set_pinned(self, idx):
        a = np.ascontiguousarray(idx, np.uint32)
        lib().orc_sim_set_pinned(self.h, ptr(a, _u32p), len(a))

    def state(self):
        x = np.zeros((self.n, 3), np.float64)
        xo = np.zeros((self.n, 3), np.float64)
        nn = np.zeros((self.n, 3), np.float64)
        lib().orc_sim_get_state(self.h, ptr(x, _dp), ptr(xo, _dp), ptr(nn, _dp))
        return x, xo, nn

    def set_state(self, x=None, xo=None, n=None):
        a = [None if v is None else np.ascontiguousarray(v, np.float32) for v in (x, xo, n)]
        lib().orc_sim_set_state(self.h, *[ptr(v, _fp) for v in a])

    def export_lbvh(self) -> dict:
        T = self.n_tris
        Tp = lib().orc_sim_n_leaves(self.h)
        ni = max(Tp - 1, 0)
        out = dict(tri_codes=np.zeros(T, np.uint32), tri_boxes=np.zeros((T, 6), np.float32),
                   sorted_codes=np.zeros(Tp, np.uint32), sorted_tris=np.zeros(Tp, np.int32),
                   child_a=np.zeros(ni, np.int32), child_b=np.zeros(ni, np.int32),
                   parent_internal=np.zeros(ni, np.int32), parent_leaf=np.zeros(Tp, np.int32),
                   internal_boxes=np.zeros((ni, 6), np.float32), leaf_boxes=np.zeros((Tp, 6), np.float32),
                   root_box=np.zeros(6, np.float32))
        o = out
        lib().orc_sim_export_lbvh(self.h, ptr(o["tri_codes"], _u32p), ptr(o["tri_boxes"], _fp),
                                  ptr(o["sorted_codes"], _u32p), ptr(o["sorted_tris"], _i32p),
                                  ptr(o["child_a"], _i32p), ptr(o["child_b"], _i32p),
                                  ptr(o["parent_internal"], _i32p), ptr(o["parent_leaf"], _i32p),
                                  ptr(o["internal_boxes"], _fp), ptr(o["leaf_boxes"], _fp), ptr(o["root_box"], _fp))
        out["n_leaves"] = Tp
        return out

    def query(self, pts):
        pts = np.ascontiguousarray(pts, np.float32)
        n = len(pts)
        leaf = np.zeros(n, np.int32)
        inside = np.zeros(n, np.int32)
        dist = np.zeros(n, np.float64)
        nrm = np.zeros((n, 3), np.float64)
        lib().orc_sim_query(self.h, ptr(pts, _fp), n, ptr(leaf, _i32p), ptr(inside, _i32p), ptr(dist, _dp),
                            ptr(nrm, _dp))
        return leaf, inside, dist, nrm

    # adjoint (FP64 reference gradient when prec = 8)
    def forward(self, nsteps: int, checkpoint_every: int = 50):
        rec = C.c_void_p()
        lib().orc_sim_forward(self.h, nsteps, checkpoint_every, C.byref(rec))
        self._rec = rec

    def backward(self, dL_dx, dL_dxo=None):
        g = np.ascontiguousarray(dL_dx, np.float64)
        go = None if dL_dxo is None else np.ascontiguousarray(dL_dxo, np.float64)
        dk = np.zeros(sum(self.n_entries), np.float64)
        ds = np.zeros(3, np.float64)
        lib().orc_sim_backward(self.h, self._rec, ptr(g, _dp), ptr(go, _dp), ptr(dk, _dp), ptr(ds, _dp))
        self._rec = None
        return dk, ds


def render(x, x_prev, faces):
    """The reference's output stage (update_vbo_pos, compute_face_normal,
    compute_vbo_normal) restated: (pos4, vertex normals, face normals)."""
    x = np.ascontiguousarray(x, np.float32)
    xp = np.ascontiguousarray(x_prev, np.float32)
    f = np.ascontiguousarray(faces, np.uint32)
    n, nf = len(x), len(f)
    pos4 = np.zeros((n, 4), np.float32)
    vn = np.zeros((n, 3), np.float32)
    fn = np.zeros((nf, 3), np.float32)
    lib().orc_render(ptr(x, _fp), ptr(xp, _fp), n, ptr(f, _u32p), nf, ptr(pos4, _fp), ptr(vn, _fp), ptr(fn, _fp))
    return pos4, vn, fn


def sh_shade(normals, rgb):
    """The reference's SH fragment shader restated at each normal: colours (n, 3)."""
    nrm = np.ascontiguousarray(normals, np.float32)
    c = np.ascontiguousarray(rgb, np.float32)
    out = np.zeros((len(nrm), 3), np.float32)
    lib().orc_sh_shade(ptr(nrm, _fp), len(nrm), ptr(c, _fp), ptr(out, _fp))
    return out


def springs_from_mesh(xyz, tris):
    """Reference spring topology (create_neigh + CSR_spring) as two SpringLists."""
    from simulator_gb300.scenes import SPRING_DTYPE, SpringList
    xyz = np.ascontiguousarray(xyz, np.float32)
    tris = np.ascontiguousarray(tris, np.uint32)
    nv, nt = len(xyz), len(tris)
    n0, n1 = C.c_int32(), C.c_int32()
    lib().orc_springs_from_mesh(ptr(xyz, _fp), nv, ptr(tris, _u32p), nt, None, None, C.byref(n0), None, None,
                                C.byref(n1))
    r0 = np.zeros(nv + 1, np.uint32)
    r1 = np.zeros(nv + 1, np.uint32)
    e0 = np.zeros(n0.value, SPRING_DTYPE)
    e1 = np.zeros(n1.value, SPRING_DTYPE)
    lib().orc_springs_from_mesh(ptr(xyz, _fp), nv, ptr(tris, _u32p), nt, ptr(r0, _u32p), e0.ctypes.data,
                                C.byref(n0), ptr(r1, _u32p), e1.ctypes.data, C.byref(n1))
    return [SpringList(r0, e0), SpringList(r1, e1)]


# --------------------------------------------------------------------------------------
# the reference's own kernels (oracle/_ref/refkern.cubin via oracle/_build/librefharness.so)
# --------------------------------------------------------------------------------------
HARNESS_PATH = os.path.join(_HERE, "_build", "librefharness.so")
CUBIN_PATH = os.path.join(_HERE, "_ref", "refkern.cubin")
_hlib = None


def refkern_available() -> bool:
    return os.path.exists(HARNESS_PATH) and os.path.exists(CUBIN_PATH)


def hlib():
    global _hlib
    if _hlib is None:
        if not refkern_available():
            raise RuntimeError("refkern not built (needs oracle/_ref/refkern.cubin and the harness)")
        L = C.CDLL(HARNESS_PATH)
        L.ref_last_error.restype = C.c_char_p
        L.ref_init.argtypes = [C.c_char_p]
        L.ref_sim_create.restype = C.c_void_p
        L.ref_sim_create.argtypes = [C.POINTER(VisgParams), _fp, C.c_int, _u32p, C.c_void_p, _u32p, C.c_void_p,
                                     _fp, _fp, C.c_int, _u32p, C.c_int]
        L.ref_sim_destroy.argtypes = [C.c_void_p]
        L.ref_sim_step.argtypes = [C.c_void_p, C.c_int]
        L.ref_sim_update_body.argtypes = [C.c_void_p, _fp, _fp]
        L.ref_sim_set_vertex.argtypes = [C.c_void_p, C.c_int, _fp]
        L.ref_sim_get_state.argtypes = [C.c_void_p, _fp, _fp, _fp]
        L.ref_sim_set_state.argtypes = [C.c_void_p, _fp, _fp, _fp]
        L.ref_sim_n_leaves.argtypes = [C.c_void_p]
        L.ref_sim_refit_race.argtypes = [C.c_void_p, C.c_int]
        L.ref_sim_refit_race.restype = C.c_longlong
        L.ref_sim_export_lbvh.argtypes = [C.c_void_p, _u32p, _fp, _u32p, _i32p, _i32p, _i32p, _i32p, _i32p, _fp,
                                          _fp, _fp]
        L.ref_render.argtypes = [_fp, _fp, C.c_int, _u32p, C.c_int, _fp, _fp, _fp]
        if L.ref_init(CUBIN_PATH.encode()) != 0:
            raise RuntimeError("refkern init failed: " + L.ref_last_error().decode())
        _hlib = L
    return _hlib


def ref_render(x, x_prev, faces):
    """The reference's own update_vbo_pos / compute_face_normal / compute_vbo_normal
    kernels on the GPU: (pos4, vertex normals, face normals)."""
    x = np.ascontiguousarray(x, np.float32)
    xp = np.ascontiguousarray(x_prev, np.float32)
    f = np.ascontiguousarray(faces, np.uint32)
    n, nf = len(x), len(f)
    pos4 = np.zeros((n, 4), np.float32)
    vn = np.zeros((n, 3), np.float32)
    fn = np.zeros((max(nf, 1), 3), np.float32)
    if hlib().ref_render(ptr(x, _fp), ptr(xp, _fp), n, ptr(f, _u32p), nf, ptr(pos4, _fp), ptr(vn, _fp),
                         ptr(fn, _fp)) != 0:
        raise RuntimeError("ref_render: " + hlib().ref_last_error().decode())
    return pos4, vn, fn[:nf]


class RefSim:
    """The reference's verlet/LBVH kernels on the GPU, driven like Simulator."""

    def __init__(self, params: VisgParams, xyz, lists, body_xyz, body_tris, body_normals=None):
        assert len(lists) == 2, "the reference has a structure and a bend list"
        L = hlib()
        self._keep = []
        xyz = np.ascontiguousarray(xyz, np.float32)
        self.n = len(xyz)
        r0 = np.ascontiguousarray(lists[0].row, np.uint32)
        r1 = np.ascontiguousarray(lists[1].row, np.uint32)
        e0 = np.ascontiguousarray(lists[0].ent)
        e1 = np.ascontiguousarray(lists[1].ent)
        bx = np.ascontiguousarray(body_xyz, np.float32)
        bt = np.ascontiguousarray(body_tris, np.uint32)
        bn = None if body_normals is None else np.ascontiguousarray(body_normals, np.float32)
        self._keep += [r0, r1, e0, e1]
        self.n_tris = len(bt)
        self.h = L.ref_sim_create(C.byref(params), ptr(xyz, _fp), self.n, ptr(r0, _u32p), e0.ctypes.data,
                                  ptr(r1, _u32p), e1.ctypes.data, ptr(bx, _fp), ptr(bn, _fp), len(bx),
                                  ptr(bt, _u32p), len(bt))
        if not self.h:
            raise RuntimeError("ref_sim_create: " + L.ref_last_error().decode())

    def _ok(self, r):
        if r != 0:
            raise RuntimeError(hlib().ref_last_error().decode())

    def close(self):
        if getattr(self, "h", None):
            hlib().ref_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n=1):
        self._ok(hlib().ref_sim_step(self.h, n))

    def refit_race(self, repair=None) -> int:
        """Internal boxes the reference's unfenced refit got wrong, over all builds so
        far; repair=True makes later builds replace them by the boxes the refit's
        definition gives (the other kernels then run on the defined tree)."""
        return int(hlib().ref_sim_refit_race(self.h, -1 if repair is None else int(bool(repair))))

    def update_body(self, xyz, normals=None):
        xyz = np.ascontiguousarray(xyz, np.float32)
        nn = None if normals is None else np.ascontiguousarray(normals, np.float32)
        self._ok(hlib().ref_sim_update_body(self.h, ptr(xyz, _fp), ptr(nn, _fp)))

    def set_vertex(self, idx, xyz):
        v = np.ascontiguousarray(xyz, np.float32)
        self._ok(hlib().ref_sim_set_vertex(self.h, idx, ptr(v, _fp)))

    def state(self):
        x, xo, n = (np.zeros((self.n, 3), np.float32) for _ in range(3))
        self._ok(hlib().ref_sim_get_state(self.h, ptr(x, _fp), ptr(xo, _fp), ptr(n, _fp)))
        return x, xo, n

    def set_state(self, x=None, xo=None, n=None):
        a = [None if v is None else np.ascontiguousarray(v, np.float32) for v in (x, xo, n)]
        self._ok(hlib().ref_sim_set_state(self.h, *[ptr(v, _fp) for v in a]))

    def export_lbvh(self) -> dict:
        T = self.n_tris
        Tp = hlib().ref_sim_n_leaves(self.h)
        ni = max(Tp - 1, 0)
        o = dict(tri_codes=np.zeros(T, np.uint32), tri_boxes=np.zeros((T, 6), np.float32),
                 sorted_codes=np.zeros(Tp, np.uint32), sorted_tris=np.zeros(Tp, np.int32),
                 child_a=np.zeros(ni, np.int32), child_b=np.zeros(ni, np.int32),
                 parent_internal=np.zeros(ni, np.int32), parent_leaf=np.zeros(Tp, np.int32),
                 internal_boxes=np.zeros((ni, 6), np.float32), leaf_boxes=np.zeros((Tp, 6), np.float32),
                 root_box=np.zeros(6, np.float32))
        self._ok(hlib().ref_sim_export_lbvh(self.h, ptr(o["tri_codes"], _u32p), ptr(o["tri_boxes"], _fp),
                                            ptr(o["sorted_codes"], _u32p), ptr(o["sorted_tris"], _i32p),
                                            ptr(o["child_a"], _i32p), ptr(o["child_b"], _i32p),
                                            ptr(o["parent_internal"], _i32p), ptr(o["parent_leaf"], _i32p),
                                            ptr(o["internal_boxes"], _fp), ptr(o["leaf_boxes"], _fp),
                                            ptr(o["root_box"], _fp)))
        o["n_leaves"] = Tp
        return o
