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


def fd_check(p, cloth, lists, body, steps, ckpt, target, entries, gamma_check=True, rel=1e-2, min_rel=1e-6):
    """GPU adjoint vs FP64 central differences on the given (list, entry) springs
    (both directed entries of the spring are perturbed together).

    The adjoint differentiates the trajectory with every step's contact set frozen
    as the forward pass found it, so a difference quotient only measures the same
    derivative if neither perturbed run changes any step's contact set.  Each
    spring's relative step starts at `rel` and is divided by 10 until both runs
    keep the unperturbed run's contact history (the oracle's contact hash), down to
    `min_rel`.  Returns (relative errors, steps used, whether the contact history
    was kept, dk, dscalar, contact counts of the unperturbed run)."""
    g = vs.Simulator(cloth.xyz, lists, None if body is None else body.xyz, None if body is None else body.tris,
                     None if body is None else body.normals, params=p, pinned=cloth.pinned)
    g.forward(steps, ckpt)
    x = g.positions()
    dk, ds = g.backward((2.0 * (x - target) / len(x)).astype(np.float32))
    g.close()
    off = np.concatenate([[0], np.cumsum([sl.n_entries for sl in lists])])
    rev = reverse_map(lists)

    def run(lst, params=p, counts=None):
        s = OracleSim(params, cloth.xyz, lst, None if body is None else body.xyz, None if body is None else body.tris,
                      None if body is None else body.normals, prec=8, pinned=cloth.pinned)
        if counts is None:
            s.step(steps)
        else:  # the unperturbed run: vertices in contact at ten points along it
            for k in range(10):
                s.step(steps // 10 if k < 9 else steps - 9 * (steps // 10))
                counts.append(int((np.abs(s.state()[2]).sum(1) > 0).sum()))
        xx = s.state()[0]
        h = s.contact_hash()
        s.close()
        return float(((xx - target) ** 2).sum() / len(xx)), h

    counts = []
    _, h0 = run(lists, counts=counts)
    errs, used, kept = [], [], []
    for l, e in entries:
        e2 = int(rev[l][e])
        k0 = float(lists[l].k[e])
        r = rel
        while True:
            up = [sl.k.copy() for sl in lists]
            dn = [sl.k.copy() for sl in lists]
            h = max(r * abs(k0), 2.0 * float(np.spacing(np.float32(k0))))
            for kk, sgn in ((up, 1.0), (dn, -1.0)):
                kk[l][e] = np.float32(k0 + sgn * h)
                kk[l][e2] = kk[l][e]
            (lu, hu), (ld, hd) = run(with_k(lists, up)), run(with_k(lists, dn))
            same = hu == h0 and hd == h0
            if same or r <= min_rel * 1.0001:
                break
            r /= 10.0
        hh = (float(up[l][e]) - float(dn[l][e])) / 2.0
        fd = (lu - ld) / (2.0 * hh)
        adj = float(dk[off[l] + e] + dk[off[l] + e2])
        errs.append(abs(adj - fd) / max(abs(fd), 1e-30))
        used.append(r)
        kept.append(same)
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
        (lu, hu), (ld, hd) = run(lists, pu), run(lists, pd)
        fd = (lu - ld) / (2.0 * hh)
        errs.append(abs(float(ds[0]) - fd) / max(abs(fd), 1e-30))
        used.append(h / gam)
        kept.append(hu == h0 and hd == h0)
    return np.array(errs), np.array(used), np.array(kept), dk, ds, counts


def test_adjoint_vs_fp64_finite_differences_small():
    cloth = scenes.grid_cloth(10, 0.5, 0.0)
    p = scenes.physics_params(4)
    lists = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0), np.random.default_rng(3), 0.2))
    target = cloth.xyz + np.float32(0.005)
    rng = np.random.default_rng(5)
    entries = [(int(l), int(rng.integers(0, lists[l].n_entries))) for l in rng.integers(0, 3, 8)]
    errs, _, _, _, _, _ = fd_check(p, cloth, lists, None, 60, 16, target, entries, rel=1e-4)
    print("relative errors:", np.array2string(errs, precision=2))
    assert errs.max() <= FD_REL


def test_adjoint_fd_through_contact_draped():
    """A 32 x 32 sheet (0.5 m) lands 5 mm below its start on a sphere (r = 0.3 m)
    and drapes over it: vertices are projected in every step from about step 30 to
    the end (400 steps, 0.2 s at 2 steps per 1e-3 s frame), so the frozen active
    set is non-empty through most of the trajectory and the projection's Jacobian
    (I - nu nu^T) and the inelastic force projection (I - n n^T) are on the path of
    every gradient.  32 seeded springs and the Verlet damping against FP64 central
    differences whose runs keep every step's contact set (the oracle's contact
    hash)."""
    cloth = scenes.grid_cloth(32, 0.5, 0.0, pin_top_corners=False)
    body = scenes.icosphere(3, 0.3, center=(0.0, -0.31, 0.0))
    p = scenes.physics_params(2)
    lists = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0)))
    perturbed = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0), np.random.default_rng(8), 0.2))
    t = vs.Simulator(cloth.xyz, perturbed, body.xyz, body.tris, body.normals, params=p)
    t.simulate(400)
    target = t.positions()
    t.close()
    rng = np.random.default_rng(32)
    entries = [(int(l), int(rng.integers(0, lists[l].n_entries))) for l in rng.integers(0, 3, 32)]
    errs, used, kept, dk, ds, counts = fd_check(p, cloth, lists, body, 400, 50, target, entries, rel=1e-3)
    print(f"draped: contacts along the run {counts}; max relative error {errs.max():.2e}, median "
          f"{np.median(errs):.2e}; steps used {sorted(set(np.round(np.log10(used)).astype(int).tolist()))} "
          f"(log10); contact history kept in {int(kept.sum())} of {len(kept)}")
    assert min(counts[1:]) > 0 and max(counts) > 20, "the sheet must stay in contact through the run"
    assert kept.all()
    assert errs.max() <= FD_REL


def test_adjoint_config4_vs_fp64_finite_differences():
    """Config 4 over its stated 0.5 s: a 128 x 128 sheet (16,384 vertices) over the
    64x64 workload's sphere (radius 0.3 m, subdivision 4, centre 0.5 m below), 1,000
    steps of 5e-4 s (2 per 1e-3 s frame: one is unstable at these stiffnesses),
    checkpoint every 50.  The sheet hangs from its two pinned corners; it reaches the
    sphere after about 0.27 s and swings across it (up to ~230 vertices projected per
    step) until about 0.43 s.  Target: the final positions of a run with per-spring stiffness
    k * exp(N(0, 0.2)) (seed 4); loss: mean squared final-position error; gradients for
    every per-spring stiffness and the Verlet damping, checked against FP64 central
    differences on 64 seeded springs whose runs keep every step's contact set (steps
    from 1e-2 relative down, by tens).  The config's 1e-6 step is reported on 16 of
    them: the sampled gradients span six orders of magnitude, and for the smallest the
    loss difference of a 1e-6 step is within the FP64 rounding noise of the
    trajectory, so that quotient is noisy (printed, not asserted)."""
    cloth = scenes.grid_cloth(128, 1.0, 0.0)
    body = scenes.icosphere(4, 0.3, center=(0.0, -0.5, 0.0))
    p = scenes.physics_params(2)
    steps = 1000
    nominal = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0)))
    perturbed = with_k(cloth.lists, spring_ks(cloth.lists, (2000.0, 1000.0, 500.0), np.random.default_rng(4), 0.2))
    t = vs.Simulator(cloth.xyz, perturbed, body.xyz, body.tris, body.normals, params=p, pinned=cloth.pinned)
    t.simulate(steps)
    target = t.positions()
    t.close()
    rng = np.random.default_rng(64)
    entries = [(int(l), int(rng.integers(0, nominal[l].n_entries))) for l in rng.integers(0, 3, 64)]
    errs, used, kept, dk, ds, counts = fd_check(p, cloth, nominal, body, steps, 50, target, entries, rel=1e-2)
    errs6, _, kept6, _, _, _ = fd_check(p, cloth, nominal, body, steps, 50, target, entries[:16], gamma_check=False,
                                        rel=1e-6)
    worst = np.argsort(errs)[-3:][::-1]
    print("config 4 worst:", [(int(w), "gamma" if w == len(entries) else entries[w], f"{errs[w]:.2e}") for w in worst])
    print(f"config 4: contacts along the run {counts}; max relative error {errs.max():.2e}, median "
          f"{np.median(errs):.2e} (64 springs, steps {sorted(set(np.round(np.log10(used[:-1])).astype(int).tolist()))} "
          f"(log10), damping at 2 ulps; contact history kept in {int(kept.sum())} of {len(kept)}); step 1e-6 on 16 "
          f"springs: max {errs6.max():.2e}, median {np.median(errs6):.2e} (history kept in {int(kept6.sum())}); "
          f"|dL/dk| max {np.abs(dk).max():.3e}, dL/dgamma {ds[0]:.3e}")
    assert max(counts) > 100 and sum(c > 0 for c in counts) >= 3, "the sheet must cross the sphere"
    assert kept.all()
    assert errs.max() <= FD_REL
