"""visg_lbvh_build_noalloc: the body LBVH build for callers that cannot allocate
device memory (their own pool owns the GPU, or an allocation at that point would
synchronise the device).  All of its temporaries live in a static device array,
so the call itself allocates nothing; this test allocates the inputs and outputs
itself (with torch) and passes them in, as such a caller would.

Checked through the C ABI, on two calls in a row (the second reuses the static
array the first one left behind), against the allocating entry point
(visg_create + visg_export_lbvh) on the same bodies: the Morton order, the
de-duplicated triangle order, the leaf count and the radix-tree links must be
identical (integer data, bit-exact).  Oversized bodies must be rejected; a body
at exactly the size limit must build; a triangle whose vertex index is out of
range must make the call report failure (n_leaves = -1) without reading outside
the vertex array; and a call must leave the device's free memory unchanged.
"""
import ctypes as C

import numpy as np
import pytest

import simulator_gb300 as vs
from simulator_gb300 import scenes
from simulator_gb300.params import reference_params

pytestmark = pytest.mark.gpu

THICKNESS = 0.003
DEPTH = 0.01


def build_noalloc(body, free_memory=None):
    """The no-alloc build of `body` through the C ABI; with `free_memory` (a list),
    the device's free memory before and after the call is appended to it."""
    import torch
    L = vs.lib()
    nv, nt = len(body.xyz), len(body.tris)
    d_xyz = torch.from_numpy(np.ascontiguousarray(body.xyz, np.float32)).cuda()
    d_nrm = None if body.normals is None else torch.from_numpy(np.ascontiguousarray(body.normals, np.float32)).cuda()
    d_tri = torch.from_numpy(np.ascontiguousarray(body.tris, np.uint32).view(np.int32)).cuda()
    codes = torch.full((nt,), -1, dtype=torch.int32, device="cuda")
    tris = torch.full((nt,), -1, dtype=torch.int32, device="cuda")
    ca = torch.zeros(max(nt - 1, 1), dtype=torch.int32, device="cuda")
    cb = torch.zeros(max(nt - 1, 1), dtype=torch.int32, device="cuda")
    nl = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    torch.cuda.synchronize()
    if free_memory is not None:
        free_memory.append(torch.cuda.mem_get_info()[0])
    rc = L.visg_lbvh_build_noalloc(d_xyz.data_ptr(), None if d_nrm is None else d_nrm.data_ptr(), nv,
                                   d_tri.data_ptr(), nt, THICKNESS, DEPTH, codes.data_ptr(), tris.data_ptr(),
                                   ca.data_ptr(), cb.data_ptr(), nl.data_ptr(), stream.cuda_stream)
    assert rc == 0, vs.STATUS.get(rc, rc)
    torch.cuda.synchronize()
    if free_memory is not None:
        free_memory.append(torch.cuda.mem_get_info()[0])
    n = int(nl.item())
    return dict(n_leaves=n, sorted_codes=codes.cpu().numpy().view(np.uint32)[:n], sorted_tris=tris.cpu().numpy()[:n],
                child_a=ca.cpu().numpy()[:max(n - 1, 0)], child_b=cb.cpu().numpy()[:max(n - 1, 0)])


def build_allocating(body):
    cloth = scenes.grid_cloth(4, 1.0, 5.0, pin_top_corners=False)
    p = reference_params(3)
    p.thickness, p.box_depth = THICKNESS, DEPTH
    s = vs.Simulator(cloth.xyz, cloth.lists, body.xyz, body.tris, body.normals, params=p)
    out = s.export_lbvh()
    s.close()
    return out


def same(a, b):
    assert a["n_leaves"] == b["n_leaves"]
    for k in ("sorted_codes", "sorted_tris", "child_a", "child_b"):
        assert np.array_equal(a[k], b[k]), k


def test_noalloc_build_matches_allocating_build_twice():
    first = scenes.icosphere(5, 0.3, (0.0, -0.5, 0.0), noise=0.02, seed=5)   # 20,480 triangles
    second = scenes.three_capsules()                                         # 19,392 triangles
    for body in (first, second):
        same(build_noalloc(body), build_allocating(body))
    # the same body again after a different one: nothing stale from the last call,
    # and the call takes no device memory (the library's static array was reserved
    # when its module loaded, before the first call)
    free = []
    same(build_noalloc(first, free), build_allocating(first))
    assert free[0] == free[1], f"free device memory changed by {free[0] - free[1]} bytes across the call"


def test_noalloc_body_at_the_size_limit():
    """Exactly VISG_NOALLOC_MAX_VERTICES vertices and VISG_NOALLOC_MAX_TRIS triangles
    (random triangles over a random point cloud, many duplicate Morton codes)."""
    rng = np.random.default_rng(11)
    nv = nt = 32768
    xyz = rng.uniform(-0.5, 0.5, size=(nv, 3)).astype(np.float32)
    tris = rng.integers(0, nv, size=(nt, 3)).astype(np.uint32)
    body = scenes.Body(xyz=xyz, tris=tris, normals=None)
    a = build_noalloc(body)
    assert a["n_leaves"] > 1000
    same(a, build_allocating(body))


def test_noalloc_rejects_an_out_of_range_vertex_index():
    """A triangle naming vertex n_vertices (one past the end): the device check
    reads vertex 0 in its place and the call reports failure; the next call with a
    good body is correct again."""
    body = scenes.icosphere(3, 0.3, (0.0, -0.5, 0.0))
    tris = body.tris.copy()
    tris[len(tris) // 2, 1] = len(body.xyz)
    bad_body = scenes.Body(xyz=body.xyz, tris=tris, normals=body.normals)
    assert build_noalloc(bad_body)["n_leaves"] == -1
    same(build_noalloc(body), build_allocating(body))


def test_noalloc_rejects_bodies_beyond_the_limit():
    import torch
    L = vs.lib()
    nt = 32769
    big = torch.zeros(3 * nt, dtype=torch.float32, device="cuda")
    out = torch.zeros(nt, dtype=torch.int32, device="cuda")
    rc = L.visg_lbvh_build_noalloc(big.data_ptr(), None, 3, big.data_ptr(), nt, THICKNESS, DEPTH, out.data_ptr(),
                                   out.data_ptr(), out.data_ptr(), out.data_ptr(), out.data_ptr(), None)
    assert rc == -1  # VISG_ERR_INVALID_ARG, nothing launched
