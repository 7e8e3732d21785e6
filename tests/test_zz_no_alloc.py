"""visg_lbvh_build_noalloc: the body LBVH build for callers that cannot allocate
device memory (their own pool owns the GPU, or an allocation at that point would
synchronise the device).  All of its temporaries live in a static device array,
so the call itself allocates nothing; this test allocates the inputs and outputs
itself (with torch) and passes them in, as such a caller would.

Checked through the C ABI, on two calls in a row (the second reuses the static
array the first one left behind), against the allocating entry point
(visg_create + visg_export_lbvh) on the same bodies: the Morton order, the
de-duplicated triangle order, the leaf count and the radix-tree links must be
identical (integer data, bit-exact).  Oversized bodies must be rejected.
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


def build_noalloc(body):
    import torch
    L = vs.lib()
    nv, nt = len(body.xyz), len(body.tris)
    d_xyz = torch.from_numpy(np.ascontiguousarray(body.xyz, np.float32)).cuda()
    d_nrm = torch.from_numpy(np.ascontiguousarray(body.normals, np.float32)).cuda()
    d_tri = torch.from_numpy(np.ascontiguousarray(body.tris, np.uint32).view(np.int32)).cuda()
    codes = torch.full((nt,), -1, dtype=torch.int32, device="cuda")
    tris = torch.full((nt,), -1, dtype=torch.int32, device="cuda")
    ca = torch.zeros(max(nt - 1, 1), dtype=torch.int32, device="cuda")
    cb = torch.zeros(max(nt - 1, 1), dtype=torch.int32, device="cuda")
    nl = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = L.visg_lbvh_build_noalloc(d_xyz.data_ptr(), d_nrm.data_ptr(), nv, d_tri.data_ptr(), nt, THICKNESS, DEPTH,
                                   codes.data_ptr(), tris.data_ptr(), ca.data_ptr(), cb.data_ptr(), nl.data_ptr(),
                                   stream.cuda_stream)
    assert rc == 0, vs.STATUS.get(rc, rc)
    torch.cuda.synchronize()
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
    # the same body again after a different one: nothing stale from the last call
    same(build_noalloc(first), build_allocating(first))


def test_noalloc_rejects_bodies_beyond_the_limit():
    import torch
    L = vs.lib()
    nt = 32769
    big = torch.zeros(3 * nt, dtype=torch.float32, device="cuda")
    out = torch.zeros(nt, dtype=torch.int32, device="cuda")
    rc = L.visg_lbvh_build_noalloc(big.data_ptr(), None, 3, big.data_ptr(), nt, THICKNESS, DEPTH, out.data_ptr(),
                                   out.data_ptr(), out.data_ptr(), out.data_ptr(), out.data_ptr(), None)
    assert rc == -1  # VISG_ERR_INVALID_ARG, nothing launched
