"""Wall and ghost particle treatments the reference ships but never runs:
boun_vel (integrator.f90:394-457, compiled, never called) and comp_ghost +
ghost_en with the moving-least-squares branch (mls.f90, not compiled).

Parity against the reference is unpinned (nothing runs them); the oracle's
restatement is pinned by identities of the formulas -- a uniform fluid
velocity U is mirrored to exactly -U on every wall row with fluid
neighbours, rows without fluid neighbours stay 0, and at the reference's
particle sizes the moment determinant is below the 1e-5 threshold, so the
MLS variant equals the Shepard one -- and the GPU matches the oracle to
1e-12 relative (FP64).
"""
import numpy as np
import pytest


def _lattice(dx=0.01, n=20, vx=0.3, vy=-0.2):
    from beachslope_gb300 import scene
    p, st, gr = scene.lattice_scene(n=n, dx=dx, jitter=0.2, seed=7)
    fl = st["tid"] == 3
    st["vx"] = np.where(fl, vx, 0.0)
    st["vy"] = np.where(fl, vy, 0.0)
    return p, st, gr


def _fluid_neighbour_rows(o, p):
    c, idx, *_ = o.neighbours(p.kmax)
    g = o.get()
    m = np.arange(p.kmax)[None, :] < c[:, None]
    has = np.array([np.any(g["tid"][idx[r][m[r]]] == 3) for r in range(len(c))])
    return g, has


@pytest.mark.parametrize("stage", ["boun_vel", "ghost", "ghost_mls"])
def test_uniform_velocity_mirrored(oracle, stage):
    p, st, gr = _lattice()
    o = oracle.Oracle(p, st, None)
    o.stage("neighbour")
    g0, has = _fluid_neighbour_rows(o, p)
    o.stage(stage)
    g = o.get()
    wall = g["tid"] <= 2
    sel = wall & has
    assert sel.sum() > 50
    np.testing.assert_allclose(g["vx"][sel], -0.3, rtol=1e-13)
    np.testing.assert_allclose(g["vy"][sel], 0.2, rtol=1e-13)
    assert np.all(g["vx"][wall & ~has] == 0.0)
    fl = ~wall
    np.testing.assert_array_equal(g["vx"][fl], g0["vx"][fl])   # fluid untouched
    if stage == "boun_vel":
        assert np.all(g["vxs"][wall] == 0.0) and np.all(g["vys"][wall] == 0.0)


def test_mls_inactive_at_reference_scale(oracle):
    """h = 1.3 dx with dx = 1 cm: every moment determinant is below 1e-5, so
    the MLS branch falls back to the Shepard weights everywhere."""
    p, st, gr = _lattice()
    fl = st["tid"] == 3
    st["vx"] = np.where(fl, np.sin(7 * st["x"]) + st["y"], 0.0)
    a = oracle.Oracle(p, st, None)
    b = oracle.Oracle(p, st, None)
    for o, s in ((a, "ghost"), (b, "ghost_mls")):
        o.stage("neighbour")
        o.stage(s)
    np.testing.assert_array_equal(a.get()["vx"], b.get()["vx"])


def test_mls_active_on_coarse_lattice(oracle):
    """dx = 0.3 m: the determinant passes the threshold and the MLS weights
    change the mirrored value of a non-uniform field."""
    p, st, gr = _lattice(dx=0.3, n=12)
    fl = st["tid"] == 3
    st["vx"] = np.where(fl, 1.0 + 2.0 * st["x"] - st["y"], 0.0)
    a = oracle.Oracle(p, st, None)
    b = oracle.Oracle(p, st, None)
    for o, s in ((a, "ghost"), (b, "ghost_mls")):
        o.stage("neighbour")
        o.stage(s)
    va, vb = a.get()["vx"], b.get()["vx"]
    assert np.any(va != vb)
    assert np.all(np.isfinite(vb))


@pytest.mark.gpu
@pytest.mark.parametrize("stage,dx,n", [("boun_vel", 0.01, 20), ("ghost", 0.01, 20), ("ghost_mls", 0.3, 12),
                                        ("ghost_mls", 0.01, 20)])
def test_ghost_gpu_matches_oracle(api, oracle, stage, dx, n):
    p, st, gr = _lattice(dx=dx, n=n)
    fl = st["tid"] == 3
    st["vx"] = np.where(fl, np.sin(5 * st["x"]) + st["y"], 0.0)
    ctx = api.Context([p], [st], [None])
    o = oracle.Oracle(p, st, None)
    ctx.prime()
    o.stage("prime")
    if stage == "boun_vel":
        ctx.boun_vel()
    else:
        ctx.ghost(use_mls=(stage == "ghost_mls"))
    o.stage(stage)
    g, r = ctx.download(), o.get()
    np.testing.assert_array_equal(g["pid"], r["pid"])
    for f in ("vx", "vy", "vxs", "vys", "tke", "nut"):
        d = np.max(np.abs(g[f] - r[f])) / max(np.max(np.abs(r[f])), 1e-300)
        assert d < 1e-12, (f, d)
