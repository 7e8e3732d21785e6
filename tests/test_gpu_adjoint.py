"""GPU adjoint (visg_forward / visg_backward) against the oracle's adjoint (float
and FP64) and against FP64 central finite differences.

The contact set of every step is frozen as the forward pass found it, so the
adjoint is the derivative of the trajectory piece the forward pass is on; the
finite differences use perturbations small enough not to change it.
"""
import numpy as np
import pytest

import simulator_gb300 as vs
from oracle.ffi import OracleSim
from simulator_gb300 import scenes
from simulator_gb300.params import reference_params

pytestmark = pytest.mark.gpu

FD_REL = 1e-3  # adjoint vs FP64 central differences, relative


def reverse_map(lists):
    """For every entry (list l, index e, i -> j) the index of its (j -> i) entry."""
    out = []
    for sl in lists:
        n = len(sl.row) - 1
        src = np.repeat(np.arange(n), np.diff(sl.row.astype(np.int64)))
        dst = sl.ent["end"].astype(np.int64)
        key = {(int(a), int(b)): k for k, (a, b) in enumerate(zip(src, dst))}
        out.append(np.array([key[(int(b), int(a))] for a, b in zip(src, dst)], np.int64))
    return out


def with_k(lists, ks):
    return [scenes.SpringList(sl.row, sl.ent, np.ascontiguousarray(k, np.float32)) for sl, k in zip(lists, ks)]


def spring_ks(lists, base, rng=None, sigma=0.0):
    """Per-entry stiffness, symmetric per undirected spring: base k of the list,
    times exp(N(0, sigma)) drawn once per spring."""
    ks = []
    for l, (sl, rv) in enumerate(zip(lists, reverse_map(lists))):
        k = np.full(sl.n_entries, base[l], np.float64)
        if rng is not None and sigma > 0:
            f = np.exp(rng.normal(0.0, sigma, sl.n_entries))
            lo = np.minimum(np.arange(sl.n_entries), rv)
            f = f[lo]  # the lower-indexed entry of each pair decides
            k = k * f
        ks.append(k.astype(np.float32))
    return ks


def test_adjoint_matches_fp64_oracle_with_contacts():
    """The differentiable forward runs in FP64 on the GPU: its trajectory, contact set
    and gradients must match the FP64 oracle's (forward + checkpointed adjoint)."""
    cloth = scenes.grid_cloth(16, 1.0, 0.0, pin_top_corners=False)
    body = scenes.icosphere(2, 0.3, center=(0.0, -0.305, 0.0))
    p = reference_params(3)
    p.list_k[:] = (100.0, 60.0, 2.0, 0.0)
    lists = with_k(cloth.lists, spring_ks(cloth.lists, (100.0, 60.0, 2.0), np.random.default_rng(0), 0.2))
    g = vs.Simulator(cloth.xyz, lists, body.xyz, body.tris, body.normals, params=p)
    o = OracleSim(p, cloth.xyz, lists, body.xyz, body.tris, body.normals, prec=8)
    steps = 80
    g.forward(steps, 16)
    o.forward(steps, 16)
    x, _, n = g.state()
    ox, _, on = o.state()
    assert np.array_equal(x, ox.astype(np.float32))  # bit-identical FP64 trajectories, rounded
    assert np.array_equal(np.abs(n).sum(1) > 0, np.abs(on).sum(1) > 0)
    assert g.count_contacts() > 0
    target = cloth.xyz + np.float32(0.01)
    dLdx = (2.0 * (x - target) / len(x)).astype(np.float32)
    dk, ds = g.backward(dLdx)
    odk, ods = o.backward(dLdx.astype(np.float64))
    scale = np.abs(odk).max()
    assert scale > 0
    err = np.abs(dk - odk).max() / scale
    print(f"GPU adjoint vs FP64 oracle adjoint: max error {err:.2e} of the largest gradient")
    assert err <= 1e-5
    assert np.allclose(ds, ods, rtol=1e-5, atol=1e-6 * np.abs(ods).max())
    # the simulator keeps the forward pass's final state
    assert np.array_equal(g.positions(), x)


def test_adjoint_matches_fp64_oracle_config_physics():
    """Damped Verlet (gamma != 1), zero spring damping, pinned corners, a body."""
    cloth = scenes.grid_cloth(40, 1.0, 0.0)
    body = scenes.icosphere(3, 0.3, center=(0.0, -0.31, 0.0))
    p = scenes.physics_params(2)
    lists = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0), np.random.default_rng(2), 0.2))
    g = vs.Simulator(cloth.xyz, lists, body.xyz, body.tris, body.normals, params=p, pinned=cloth.pinned)
    o = OracleSim(p, cloth.xyz, lists, body.xyz, body.tris, body.normals, prec=8, pinned=cloth.pinned)
    g.forward(200, 50)
    o.forward(200, 50)
    x = g.positions()
    assert np.array_equal(x, o.state()[0].astype(np.float32))
    target = cloth.xyz + np.float32(0.01)
    dLdx = (2.0 * (x - target) / len(x)).astype(np.float32)
    dk, ds = g.backward(dLdx)
    odk, ods = o.backward(dLdx.astype(np.float64))
    err = np.abs(dk - odk).max() / np.abs(odk).max()
    print(f"config physics: dk max error {err:.2e} of the largest; dscalar {ds} vs {ods}; contacts "
          f"{g.count_contacts()}")
    assert err <= 1e-5
    assert np.allclose(ds, ods, rtol=1e-5, atol=1e-7 * np.abs(ods).max())


def fd_check(p, cloth, lists, body, steps, ckpt, target, entries, gamma_check=True, rel=1e-4):
    """GPU adjoint vs FP64 central differences on the given (list, entry) springs
    (both directed entries of the spring are perturbed together)."""
    g = vs.Simulator(cloth.xyz, lists, None if body is None else body.xyz, None if body is None else body.tris,
                     None if body is None else body.normals, params=p, pinned=cloth.pinned)
    g.forward(steps, ckpt)
    x = g.positions()
    dk, ds = g.backward((2.0 * (x - target) / len(x)).astype(np.float32))
    off = np.concatenate([[0], np.cumsum([sl.n_entries for sl in lists])])
    rev = reverse_map(lists)

    def loss(lst, params=p):
        s = OracleSim(params, cloth.xyz, lst, None if body is None else body.xyz, None if body is None else body.tris,
                      None if body is None else body.normals, prec=8, pinned=cloth.pinned)
        s.step(steps)
        xx = s.state()[0]
        s.close()
        return float(((xx - target) ** 2).sum() / len(xx))

    errs = []
    for l, e in entries:
        e2 = int(rev[l][e])
        base = [sl.k.copy() for sl in lists]
        up = [k.copy() for k in base]
        dn = [k.copy() for k in base]
        k0 = float(base[l][e])
        h = max(rel * abs(k0), 2.0 * float(np.spacing(np.float32(k0))))
        for kk, sgn in ((up, 1.0), (dn, -1.0)):
            kk[l][e] = np.float32(k0 + sgn * h)
            kk[l][e2] = kk[l][e]
        hh = (float(up[l][e]) - float(dn[l][e])) / 2.0
        fd = (loss(with_k(lists, up)) - loss(with_k(lists, dn))) / (2.0 * hh)
        adj = float(dk[off[l] + e] + dk[off[l] + e2])
        errs.append(abs(adj - fd) / max(abs(fd), 1e-30))
    if gamma_check:
        pu, pd = vs.VisgParams(), vs.VisgParams()
        for q in (pu, pd):
            for f, _ in vs.VisgParams._fields_:
                setattr(q, f, getattr(p, f))
        # gamma compounds over every step (the loss is strongly curved in it: the
        # central difference is 21% off at a 1e-4 step, 2e-3 at 1e-5), so its (large)
        # gradient is differenced with a step of two float ulps (~1.2e-7)
        gam = p.verlet_damping
        h = 2.0 * float(np.spacing(np.float32(gam)))
        pu.verlet_damping, pd.verlet_damping = float(np.float32(gam + h)), float(np.float32(gam - h))
        hh = (float(np.float32(gam + h)) - float(np.float32(gam - h))) / 2.0
        fd = (loss(lists, pu) - loss(lists, pd)) / (2.0 * hh)
        errs.append(abs(float(ds[0]) - fd) / max(abs(fd), 1e-30))
    return np.array(errs), dk, ds


def test_adjoint_vs_fp64_finite_differences_small():
    cloth = scenes.grid_cloth(10, 0.5, 0.0)
    p = scenes.physics_params(4)
    lists = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0), np.random.default_rng(3), 0.2))
    target = cloth.xyz + np.float32(0.005)
    rng = np.random.default_rng(5)
    entries = [(int(l), int(rng.integers(0, lists[l].n_entries))) for l in rng.integers(0, 3, 8)]
    errs, _, _ = fd_check(p, cloth, lists, None, 60, 16, target, entries)
    print("relative errors:", np.array2string(errs, precision=2))
    assert errs.max() <= FD_REL


def test_adjoint_config4_vs_fp64_finite_differences():
    """128 x 128 sheet (16,384 vertices) over the 64x64 workload's sphere (radius
    0.3 m, subdivision 4, centre 0.5 m below), 500 steps, checkpoint every 50.
    Target: the final positions of a run with per-spring stiffness k * exp(N(0, 0.2))
    (seed 4); loss: mean squared final-position error; gradients for every
    per-spring stiffness and the Verlet damping, checked against FP64 central
    differences on 64 seeded springs.  The sampled gradients span six orders of
    magnitude (1e-16 .. 3e-10); for the smallest, the loss difference of a 1e-6 or
    1e-4 step is within a few thousand ulps of the loss, so the difference quotient
    itself is noisy (1e-2 .. 1e0; the 1e-6 result is printed).  The loss is linear in
    one spring's stiffness to that order, so the assertion uses a 1e-2 step
    (truncation error measured below 1e-4)."""
    cloth = scenes.grid_cloth(128, 1.0, 0.0)
    body = scenes.icosphere(4, 0.3, center=(0.0, -0.5, 0.0))
    p = scenes.physics_params(2)
    nominal = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0)))
    perturbed = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0), np.random.default_rng(4), 0.2))
    t = vs.Simulator(cloth.xyz, perturbed, body.xyz, body.tris, body.normals, params=p, pinned=cloth.pinned)
    t.simulate(500)
    target = t.positions()
    t.close()
    rng = np.random.default_rng(64)
    entries = [(int(l), int(rng.integers(0, nominal[l].n_entries))) for l in rng.integers(0, 3, 64)]
    errs, dk, ds = fd_check(p, cloth, nominal, body, 500, 50, target, entries, rel=1e-2)
    errs6, _, _ = fd_check(p, cloth, nominal, body, 500, 50, target, entries[:16], gamma_check=False, rel=1e-6)
    worst = np.argsort(errs)[-3:][::-1]
    print("config 4 worst:", [(int(w), "gamma" if w == len(entries) else entries[w], f"{errs[w]:.2e}") for w in worst])
    print(f"config 4: max relative error {errs.max():.2e}, median {np.median(errs):.2e} "
          f"(64 springs at step 1e-2, damping at 2 ulps); step 1e-6 on 16 springs: max {errs6.max():.2e}, "
          f"median {np.median(errs6):.2e}; |dL/dk| max {np.abs(dk).max():.3e}, dL/dgamma {ds[0]:.3e}")
    assert errs.max() <= FD_REL
