"""Collision shifts the reference compiles but never calls: coll_pos_shift
and coll_shift (part_shift.f90:193-410).

Parity against the reference is unpinned (nothing runs them).  The oracle's
restatement is pinned by an independent numpy evaluation of the routines
over the oracle's own neighbour lists and by identities (no overlap moves
nothing; a uniform pore velocity has no approaching pairs); the GPU matches
the oracle to 1e-12 relative (FP64).
"""
import numpy as np
import pytest


def _scene(kind="lattice"):
    from beachslope_gb300 import scene
    if kind == "lattice":
        p, st, gr = scene.lattice_scene(n=20, dx=0.01, jitter=0.2, seed=7)
        gr = None
    else:
        p, st, gr = scene.beach_scene(dx=0.02)
    fl = st["tid"] == 3
    rng = np.random.default_rng(3)
    st["vx"] = np.where(fl, 0.2 + 0.3 * np.sin(9 * st["x"]) + 0.05 * rng.standard_normal(len(fl)), 0.0)
    st["vy"] = np.where(fl, -0.1 + 0.2 * np.cos(7 * st["y"]), 0.0)
    return p, st, gr


def _spacings(p, f=1.1):
    return 0.5 * p.dl * f, 0.5 * p.dl * f, 0.5 * p.dl, 0.5 * p.dl


def _numpy_shift(g, counts, idx, dist, mode, prx, pry, brx, bry):
    """part_shift.f90:193-410 evaluated pair by pair in numpy."""
    n = len(g["x"])
    out = np.zeros((n, 2))
    elig = (counts > 0) & (g["gradvx"] >= 0.70) & (g["tid"] == 3) & ((g["flags"] & 4) == 0)
    for i in np.nonzero(elig)[0]:
        js, ds = idx[i, :counts[i]], dist[i, :counts[i]]
        phi_i, phi_j = g["porosity"][i], g["porosity"][js]
        for ax, (pr, br) in enumerate(((prx, brx), (pry, bry))):
            dcol = pr * (1.0 / np.sqrt(phi_i)) + np.where(g["tid"][js] == 3, pr, br) * (1.0 / np.sqrt(phi_j))
            rel = (g["y"][i] - g["y"][js]) if ax else (g["x"][i] - g["x"][js])
            if mode == 0:
                term = np.where(ds < dcol, (-1.0 * (g["mass"][js] * 1.0 * (ds - dcol))) * (rel / ds), 0.0)
            else:
                t3 = (g["x"][i] - g["x"][js]) * (g["vx"][i] * (1.0 / phi_i) - g["vx"][js] * (1.0 / phi_j)) + \
                     (g["y"][i] - g["y"][js]) * (g["vy"][i] * (1.0 / phi_i) - g["vy"][js] * (1.0 / phi_j))
                term = np.where((ds < dcol) & (t3 < 0.0), (-1.0 * (g["mass"][js] * 1.0 * t3)) * (rel / (ds * ds)), 0.0)
            out[i, ax] = term.sum() / (g["mass"][i] + g["mass"][js].sum())
    return out, elig


@pytest.mark.parametrize("mode", [0, 1])
def test_collision_oracle_matches_numpy(oracle, mode):
    p, st, gr = _scene("beach")
    o = oracle.Oracle(p, st, gr)
    o.stage("prime")
    g0 = o.get()
    counts, idx, dist, *_ = o.neighbours(p.kmax)
    sp = _spacings(p)
    want, elig = _numpy_shift(g0, counts, idx, dist, mode, *sp)
    assert elig.sum() > 100
    o.collision_shift(mode, *sp)
    g = o.get()
    got = np.c_[g["xs"], g["ys"]] if mode == 0 else np.c_[g["vxs"], g["vys"]]
    assert np.any(want != 0.0)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-18)
    if mode == 0:
        mv = elig
        np.testing.assert_array_equal(g["x"][mv], g0["x"][mv] + g["xs"][mv])
        np.testing.assert_array_equal(g["x"][~mv], g0["x"][~mv])
    else:
        fl = (g["tid"] == 3) & ((g["flags"] & 4) == 0)
        np.testing.assert_array_equal(g["vx"][fl], g0["vx"][fl] + g["vxs"][fl] * g["porosity"][fl])
        np.testing.assert_array_equal(g["vx"][~fl], g0["vx"][~fl])


def test_collision_identities_oracle(oracle):
    # collision distance below every pair distance: nothing moves, shifts 0
    p, st, gr = _scene("lattice")
    o = oracle.Oracle(p, st, None)
    o.stage("prime")
    g0 = o.get()
    o.collision_shift(0, 1e-9, 1e-9, 1e-9, 1e-9)
    g = o.get()
    np.testing.assert_array_equal(g["x"], g0["x"])
    assert np.all(g["xs"] == 0.0) and np.all(g["ys"] == 0.0)
    # a uniform pore velocity has no approaching pair: velocities unchanged
    st["vx"] = np.where(st["tid"] == 3, 0.3, 0.0)
    st["vy"] = np.where(st["tid"] == 3, -0.2, 0.0)
    st["vx"][st["tid"] <= 2] = 0.3
    st["vy"][st["tid"] <= 2] = -0.2
    o = oracle.Oracle(p, st, None)
    o.stage("prime")
    g0 = o.get()
    o.collision_shift(1, *_spacings(p, 1.5))
    g = o.get()
    assert np.all(g["vxs"] == 0.0) and np.all(g["vys"] == 0.0)
    np.testing.assert_array_equal(g["vx"], g0["vx"])


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["lattice", "beach"])
@pytest.mark.parametrize("mode", [0, 1])
def test_collision_gpu_matches_oracle(api, oracle, kind, mode):
    p, st, gr = _scene(kind)
    ctx = api.Context([p], [st], [gr])
    o = oracle.Oracle(p, st, gr)
    ctx.prime()
    o.stage("prime")
    sp = _spacings(p)
    ctx.collision_shift(mode, *sp)
    o.collision_shift(mode, *sp)
    g, r = ctx.download(), o.get()
    np.testing.assert_array_equal(g["pid"], r["pid"])
    fields = ("xs", "ys", "x", "y") if mode == 0 else ("vxs", "vys", "vx", "vy")
    for f in fields:
        d = np.max(np.abs(g[f] - r[f])) / max(np.max(np.abs(r[f])), 1e-300)
        assert d < 1e-12, (f, d)
    assert np.any(r[fields[0]] != 0.0)
