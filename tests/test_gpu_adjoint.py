"""GPU adjoint (visg_forward / visg_backward) against the oracle's adjoint (float
and FP64) and against FP64 central finite differences.

The contact set of every step is frozen as the forward pass found it, so the
adjoint is the derivative of the piece of the trajectory the forward pass is on.
Through resting contact no finite perturbation stays on that piece (see fd_check),
so there the differences are taken on runs that replay the recorded contact
history.
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
    fc = g.forward_contacts()  # the frozen active set, step by step
    assert fc[-1] == g.count_contacts() and (fc > 0).sum() > 10
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


def fd_check(p, cloth, lists, body, steps, ckpt, target, entries, gamma_check=True, rel=1e-2, replay=False):
    """GPU adjoint vs FP64 central differences on the given (list, entry) springs
    (both directed entries of the spring are perturbed together) and the Verlet
    damping.

    The adjoint differentiates the trajectory with every step's contact set frozen as
    the forward pass found it.  A vertex resting on the body sits exactly on its
    triangle's plane (the inelastic response removes the normal force), so whether it
    is projected again is decided by rounding, and any change of a parameter, even by
    one float ulp, flips some of those decisions: through resting contact the
    trajectory jumps at every perturbation.  With `replay` the perturbed runs replay
    the unperturbed run's contact history (the oracle applies the recorded
    projections by the branch's own formula, x' = x* - ((x* - v0) . n) n) instead of
    deciding contacts, so the quotients are derivatives of the piece of the trajectory
    the adjoint differentiates.  Returns (relative errors, dk, dscalar, counts, fd):
    counts = vertices in contact at ten points of the unperturbed run (without
    replay), then the number of GPU forward steps whose frozen active set was
    non-empty; fd = the difference quotients."""
    g = vs.Simulator(cloth.xyz, lists, None if body is None else body.xyz, None if body is None else body.tris,
                     None if body is None else body.normals, params=p, pinned=cloth.pinned)
    g.forward(steps, ckpt)
    x = g.positions()
    fwd = g.forward_contacts()
    dk, ds = g.backward((2.0 * (x - target) / len(x)).astype(np.float32))
    g.close()
    off = np.concatenate([[0], np.cumsum([sl.n_entries for sl in lists])])
    rev = reverse_map(lists)

    def sim(lst, params=p):
        return OracleSim(params, cloth.xyz, lst, None if body is None else body.xyz,
                         None if body is None else body.tris, None if body is None else body.normals, prec=8,
                         pinned=cloth.pinned)

    base = sim(lists)
    counts = []
    record = base.record_contacts(steps) if replay else None
    if not replay:
        for k in range(10):
            base.step(steps // 10 if k < 9 else steps - 9 * (steps // 10))
            counts.append(int((np.abs(base.state()[2]).sum(1) > 0).sum()))
    base.close()
    counts.append(int((fwd > 0).sum()))  # last: forward steps with a non-empty active set

    def loss(lst, params=p):
        s = sim(lst, params)
        if replay:
            s.step_forced(record)
        else:
            s.step(steps)
        xx = s.state()[0]
        s.close()
        return float(((xx - target) ** 2).sum() / len(xx))

    errs, fds = [], []
    for l, e in entries:
        e2 = int(rev[l][e])
        k0 = float(lists[l].k[e])
        up = [sl.k.copy() for sl in lists]
        dn = [sl.k.copy() for sl in lists]
        h = max(rel * abs(k0), 2.0 * float(np.spacing(np.float32(k0))))
        for kk, sgn in ((up, 1.0), (dn, -1.0)):
            kk[l][e] = np.float32(k0 + sgn * h)
            kk[l][e2] = kk[l][e]
        hh = (float(up[l][e]) - float(dn[l][e])) / 2.0
        fd = (loss(with_k(lists, up)) - loss(with_k(lists, dn))) / (2.0 * hh)
        adj = float(dk[off[l] + e] + dk[off[l] + e2])
        errs.append(abs(adj - fd) / max(abs(fd), 1e-30))
        fds.append(fd)
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
        fds.append(fd)
    return np.array(errs), dk, ds, counts, np.array(fds)


def test_adjoint_vs_fp64_finite_differences_small():
    cloth = scenes.grid_cloth(10, 0.5, 0.0)
    p = scenes.physics_params(4)
    lists = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0), np.random.default_rng(3), 0.2))
    target = cloth.xyz + np.float32(0.005)
    rng = np.random.default_rng(5)
    entries = [(int(l), int(rng.integers(0, lists[l].n_entries))) for l in rng.integers(0, 3, 8)]
    errs, _, _, _, _ = fd_check(p, cloth, lists, None, 60, 16, target, entries, rel=1e-4)
    print("relative errors:", np.array2string(errs, precision=2))
    assert errs.max() <= FD_REL


def test_adjoint_fd_through_contact_draped():
    """A 32 x 32 sheet (0.5 m) lands 5 mm below its start on a sphere (r = 0.3 m) and
    drapes over it: 400 steps (0.1 s at 4 steps per 1e-3 s frame), with vertices
    projected onto the sphere in most of them, so the projection's Jacobian
    (I - nu nu^T), the inelastic force projection (I - n n^T) and the velocity reset
    of every projected vertex are on the path of every gradient.  Target: the final
    positions of a run with per-spring stiffness k * exp(N(0, 0.2)).  64 seeded
    springs and the Verlet damping against FP64 central differences (3e-3 relative)
    of runs that replay the unperturbed run's contact history.  The sampled spring
    gradients span five orders of magnitude; a spring whose gradient is below 1e-4 of
    the largest has a loss difference at the FP64 noise floor of the trajectory, so
    it is held to 1e-6 of the largest gradient in absolute terms instead (counted and
    printed); the others, and the damping, to 1e-3 relative."""
    cloth = scenes.grid_cloth(32, 0.5, 0.0, pin_top_corners=False)
    body = scenes.icosphere(3, 0.3, center=(0.0, -0.31, 0.0))
    p = scenes.physics_params(4)
    steps = 400
    lists = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0)))
    perturbed = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0), np.random.default_rng(8), 0.2))
    t = OracleSim(p, cloth.xyz, perturbed, body.xyz, body.tris, body.normals, prec=8)
    t.step(steps)
    target = t.state()[0].astype(np.float32)
    t.close()
    rng = np.random.default_rng(32)
    entries = [(int(l), int(rng.integers(0, lists[l].n_entries))) for l in rng.integers(0, 3, 64)]
    errs, dk, ds, counts, fds = fd_check(p, cloth, lists, body, steps, 50, target, entries, rel=3e-3, replay=True)
    scale = np.abs(fds[:-1]).max()
    big = np.append(np.abs(fds[:-1]) >= 1e-4 * scale, True)  # the damping is held to the relative bar
    absolute = errs[~big] * np.abs(fds[~big]) / scale
    print(f"draped: forward steps with a non-empty active set {counts[-1]} of {steps}; max relative error "
          f"{errs[big].max():.2e}, median {np.median(errs[big]):.2e} ({int(big.sum()) - 1} springs + damping); "
          f"{int((~big).sum())} springs with gradients below 1e-4 of the largest: max error "
          f"{absolute.max() if len(absolute) else 0.0:.1e} of the largest; |dL/dk| max {np.abs(dk).max():.3e}, "
          f"dL/dgamma {ds[0]:.3e}")
    assert counts[-1] > 200, "non-empty frozen active set in most forward steps"
    assert errs[big].max() <= FD_REL
    assert len(absolute) == 0 or absolute.max() <= 1e-6


def config4(steps, substeps=4):
    """Config 4's scene: a 128 x 128 sheet (16,384 vertices, two pinned corners) over
    the 64x64 workload's sphere (radius 0.3 m, subdivision 4, centre 0.5 m below),
    with a stiffness per spring; the target is the final state of a run with
    per-spring stiffness k * exp(N(0, 0.2)) (seed 4).  At 4 steps per 1e-3 s frame:
    at 2 the stiffest perturbed springs pass the explicit step's stability limit and
    the target run blows up."""
    cloth = scenes.grid_cloth(128, 1.0, 0.0)
    body = scenes.icosphere(4, 0.3, center=(0.0, -0.5, 0.0))
    p = scenes.physics_params(substeps)
    nominal = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0)))
    perturbed = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0), np.random.default_rng(4), 0.2))
    t = OracleSim(p, cloth.xyz, perturbed, body.xyz, body.tris, body.normals, prec=8, pinned=cloth.pinned)
    t.step(steps)
    target = t.state()[0].astype(np.float32)
    t.close()
    return cloth, body, p, nominal, target


def test_adjoint_config4_vs_fp64_finite_differences():
    """Config 4 up to the sheet's first contact: 0.25 s (1,000 steps, checkpoint every
    50).  Gradients for every per-spring stiffness and the Verlet damping; 64 seeded
    springs and the damping against FP64 central differences (1e-2 relative for the
    springs: the loss is linear in one spring's stiffness to that order).  The
    config's 1e-6 step is reported on 16 of them: the sampled gradients span six
    orders of magnitude, and for the smallest the loss difference of a 1e-6 step is
    within the FP64 rounding noise of the trajectory (printed, not asserted)."""
    steps = 1000
    cloth, body, p, nominal, target = config4(steps)
    rng = np.random.default_rng(64)
    entries = [(int(l), int(rng.integers(0, nominal[l].n_entries))) for l in rng.integers(0, 3, 64)]
    errs, dk, ds, counts, _ = fd_check(p, cloth, nominal, body, steps, 50, target, entries, rel=1e-2)
    errs6, _, _, _, _ = fd_check(p, cloth, nominal, body, steps, 50, target, entries[:16], gamma_check=False,
                                 rel=1e-6)
    worst = np.argsort(errs)[-3:][::-1]
    print("config 4 (0.25 s) worst:", [(int(w), "gamma" if w == len(entries) else entries[w], f"{errs[w]:.2e}")
                                       for w in worst])
    print(f"config 4 (0.25 s): contacts along the run {counts[:10]}; max relative error {errs.max():.2e}, median "
          f"{np.median(errs):.2e} (64 springs at step 1e-2, damping at 2 ulps); step 1e-6 on 16 springs: max "
          f"{errs6.max():.2e}, median {np.median(errs6):.2e}; |dL/dk| max {np.abs(dk).max():.3e}, "
          f"dL/dgamma {ds[0]:.3e}")
    assert errs.max() <= FD_REL


def test_adjoint_config4_full_duration():
    """Config 4 over its stated 0.5 s (2,000 steps): the sheet swings across the
    sphere from about 0.27 s to 0.43 s.  Through that episode the frozen-active-set
    derivative grows by about seven orders of magnitude (projected vertices lose
    their velocity every step and the final positions become exponentially sensitive
    to the stiffnesses), so no finite-difference step both resolves the loss change
    and stays in the linear range (replayed differences at 1e-2 and 1e-4 relative
    both miss by O(1)).  What is asserted is that two independent implementations of
    the same derivative agree: the GPU adjoint (FP64 forward on the device) and the
    FP64 oracle's checkpointed adjoint, to 1e-5 of the largest gradient."""
    steps = 2000
    cloth, body, p, nominal, target = config4(steps)
    g = vs.Simulator(cloth.xyz, nominal, body.xyz, body.tris, body.normals, params=p, pinned=cloth.pinned)
    g.forward(steps, 50)
    x = g.positions()
    active = g.forward_contacts()
    dLdx = (2.0 * (x - target) / len(x)).astype(np.float32)
    dk, ds = g.backward(dLdx)
    g.close()
    o = OracleSim(p, cloth.xyz, nominal, body.xyz, body.tris, body.normals, prec=8, pinned=cloth.pinned)
    o.forward(steps, 50)
    assert np.array_equal(x, o.state()[0].astype(np.float32))
    odk, ods = o.backward(dLdx.astype(np.float64))
    o.close()
    err = np.abs(dk - odk).max() / np.abs(odk).max()
    print(f"config 4 (0.5 s): forward steps with a non-empty active set {int((active > 0).sum())} of {steps} (at "
          f"most {int(active.max())} vertices); |dL/dk| max {np.abs(odk).max():.3e}; GPU vs FP64 oracle adjoint "
          f"{err:.2e} of the largest; dL/dgamma {ds[0]:.4e} vs {ods[0]:.4e}")
    assert (active > 0).sum() > 300
    assert np.isfinite(dk).all() and err <= 1e-5
    assert abs(ds[0] - ods[0]) <= 1e-5 * abs(ods[0])
