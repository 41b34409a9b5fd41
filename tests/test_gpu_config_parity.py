"""Parity at the configured sizes: the CUDA library (through the C-ABI)
against the oracle on the workloads the benchmarks run, and the mixed form
against the FP64 drop-in on the standalone 1 M-particle search + PPE.

* 182 k particles (the solitary-wave beach at dx = 2.5 mm): two production
  steps (main.f90:199-272) of the FP64 drop-in and of the mixed form, each
  against the oracle's FP64 step from the same initial state, both solving
  the PPE to 1e-12.
* 13 k particles (dx = 10 mm) over 2000 steps of the FP64 drop-in against
  the oracle, compared every 100 steps (long-horizon drift).
* 1 M-particle jittered lattice: neighbour sets of the two precision forms
  identical, PPE with a seeded N(0,1) source solved to 1e-8 by both, pressure
  rel-L2 between them stated and bounded.

Tolerances are written in each assert.  Particle order, cell keys, neighbour
counts and neighbour sets are bit-exact between the FP64 drop-in and the
oracle; the stored pair distances too on the same positions, and within
1e-12 relative after a step (the positions then differ in the last bits).
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def relL2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def by_pid(g, r):
    """Rows of g and r paired by particle id (both hold the same ids)."""
    og, orr = np.argsort(g["pid"]), np.argsort(r["pid"])
    assert np.array_equal(g["pid"][og], r["pid"][orr])
    return og, orr


def _neighbours_equal(ctx, o, kmax, exact_dist=True):
    """Counts and neighbour sets bit-exact; the stored pair distances too
    when both codes hold the same positions, else within 1e-12 relative (the
    positions after a step differ in the last bits)."""
    cg, ig, dg, *_ = ctx.neighbours()
    co, io, do, *_ = o.neighbours(kmax)
    np.testing.assert_array_equal(cg, co)
    m = np.arange(kmax)[None, :] < co[:, None]
    np.testing.assert_array_equal(ig[m], io[m])
    if exact_dist:
        np.testing.assert_array_equal(dg[m], do[m])
    else:
        assert np.max(np.abs(dg[m] - do[m]) / do[m]) <= 1e-12
    return float(co.mean())


def test_config2_scale_steps_vs_oracle(api, oracle):
    """182 k particles, two production steps: FP64 drop-in and mixed form
    against the oracle (every stage of the reference step: search.f90,
    porous.f90, turbulence.f90, integrator.f90, isph.f90, scalar.f90,
    part_shift.f90)."""
    from beachslope_gb300 import abi, scene
    p, st, gr = scene.beach_scene(dx=0.0025)
    p.ppe_tol = 1e-12
    p.ppe_maxit = 20000
    pm = abi.Params.from_buffer_copy(p)
    pm.precision = abi.PREC_MIXED
    g64 = api.Context([p], [st], [gr], tuning="auto")
    gmx = api.Context([pm], [st], [gr], tuning="auto")
    o = oracle.Oracle(p, st, gr)
    t0 = time.time()
    o.stage("prime")
    for c in (g64, gmx):
        c.prime()
    kbar = _neighbours_equal(g64, o, p.kmax)
    for k in range(2):
        o.step(1)
        g64.step(1)
        gmx.step(1)
        r, g, m = o.get(), g64.download(), gmx.download()
        # FP64 drop-in: particle order, cell keys and neighbour lists bit-exact
        np.testing.assert_array_equal(g["pid"], r["pid"])
        np.testing.assert_array_equal(g["cell"], r["cell"])
        np.testing.assert_array_equal(g["flags"], r["flags"])
        _neighbours_equal(g64, o, p.kmax, exact_dist=False)
        e64 = {f: relL2(g[f], r[f]) for f in ("p", "vx", "vy", "con", "nut")}
        dxm = float(max(np.max(np.abs(g["x"] - r["x"])), np.max(np.abs(g["y"] - r["y"]))))
        og, orr = by_pid(m, r)
        emx = {f: relL2(m[f][og], r[f][orr]) for f in ("p", "vx", "vy", "con")}
        print(f"step {k + 1}: n={len(r['x'])} K={kbar:.1f} fp64 vs oracle {e64} max|dx| {dxm:.2e}; "
              f"mixed vs oracle {emx}")
        assert e64["p"] <= 1e-8, e64
        assert e64["vx"] <= 1e-9 and e64["vy"] <= 1e-9, e64
        assert e64["con"] <= 1e-12 and e64["nut"] <= 1e-9, e64
        assert dxm <= 1e-12, dxm
        # the mixed form against the FP64 oracle (accuracy bar: p within 1e-6
        # for one step from the same state; the second step carries the first
        # step's position differences: measured 5.8e-8, then 1.2e-6; the
        # velocities carry the FP32 pair sums of the sweeps: 3.8e-7 / 1.0e-6
        # rel-L2 after one step)
        assert emx["p"] <= (1e-6 if k == 0 else 5e-6), emx
        assert emx["vx"] <= 5e-6 and emx["vy"] <= 5e-6, emx
        assert emx["con"] <= 1e-9, emx
    assert g64.info()["err_bits"] == 0 and gmx.info()["err_bits"] == 0
    assert g64.info()["ppe_relres"] <= 1e-11
    print(f"oracle + GPU wall {time.time() - t0:.1f} s")


def test_config1_long_horizon_vs_oracle(api, oracle):
    """dx = 10 mm (13 k particles), 2000 production steps of the FP64 drop-in
    and of the oracle from the same initial state (PPE to 1e-12 in both),
    compared every 100 steps.  The two codes sum in different orders, so the
    trajectories separate slowly (measured on a GB300: positions 1e-12 m
    after 200 steps, 1.4e-8 m after 2000, i.e. 1.4e-6 of the 10 mm spacing;
    pressure within 2e-9, velocities within 4e-8 rel-L2); the bounds below
    hold the drift well below the step-to-step change of the fields."""
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.01)
    p.ppe_tol = 1e-12
    p.ppe_maxit = 20000
    ctx = api.Context([p], [st], [gr], tuning="auto")
    o = oracle.Oracle(p, st, gr)
    ctx.prime()
    o.stage("prime")
    t0 = time.time()
    rows = []
    for k in range(20):
        ctx.step(100)
        o.step(100)
        g, r = ctx.download(), o.get()
        og, orr = by_pid(g, r)
        reorder = int(np.sum(g["pid"] != r["pid"]))
        e = {f: relL2(g[f][og], r[f][orr]) for f in ("p", "vx", "vy", "con")}
        dxm = float(max(np.max(np.abs(g["x"][og] - r["x"][orr])), np.max(np.abs(g["y"][og] - r["y"][orr]))))
        rows.append((100 * (k + 1), e, dxm, reorder))
        print(f"step {100 * (k + 1):5d}: p {e['p']:.2e} vx {e['vx']:.2e} vy {e['vy']:.2e} con {e['con']:.2e} "
              f"max|dx| {dxm:.2e} m, rows ordered differently {reorder}")
    print(f"wall {time.time() - t0:.1f} s")
    assert ctx.info()["err_bits"] == 0
    gi, oi = ctx.info(), o.info()
    assert gi["t"] == pytest.approx(oi["t"], rel=1e-12)
    for step, e, dxm, reorder in rows:
        assert e["p"] <= 1e-6, (step, e)
        assert e["vx"] <= 1e-6 and e["vy"] <= 1e-6, (step, e)
        assert e["con"] <= 1e-9, (step, e)
        assert dxm <= 1e-7, (step, dxm)   # 1e-5 of the particle spacing
    # within the first 100 steps the order of every row is the oracle's
    assert rows[0][3] == 0


def test_config3_1m_mixed_vs_fp64(api):
    """1000 x 1000 jittered lattice, free surface on the top row, walls on
    three sides, seeded N(0,1) source: search + assembly + PPE to 1e-8 in
    both precision forms.  Neighbour sets identical; pressure rel-L2 of the
    mixed form against the FP64 drop-in at most 1e-6 at 1e-8, and at most
    1e-7 when both solve to 1e-12 (what is left is the mixed form's own
    arithmetic: FP32 pair values in the assembly; measured 2.9e-8)."""
    from beachslope_gb300 import abi, scene
    res = {}
    for tol in (1e-8, 1e-12):
        xs, nb = {}, {}
        for prec in (abi.PREC_FP64, abi.PREC_MIXED):
            p, st, gr = scene.lattice_scene(n=1000, dx=1e-3)
            p.precision = prec
            p.ppe_tol = tol
            p.ppe_maxit = 20000
            ctx = api.Context([p], [st], [None], tuning="auto")
            ctx.search()
            c, idx, *_ = ctx.neighbours()
            nb[prec] = (c, idx)
            ctx.porosity()
            ctx.int_vel()
            ctx.ppe_assemble()
            b = np.random.default_rng(20261203).standard_normal(len(c))
            ctx.set_rhs(b)
            ctx.ppe_solve()
            inf = ctx.info()
            assert inf["ppe_relres"] <= tol * 1.01, (prec, tol, inf)
            assert inf["err_bits"] == 0
            xs[prec] = ctx.download(full=False)["p"]
            ctx.close()
        c64, i64 = nb[abi.PREC_FP64]
        cmx, imx = nb[abi.PREC_MIXED]
        np.testing.assert_array_equal(c64, cmx)
        m = np.arange(i64.shape[1])[None, :] < c64[:, None]
        np.testing.assert_array_equal(i64[m], imx[m])
        res[tol] = relL2(xs[abi.PREC_MIXED], xs[abi.PREC_FP64])
    print(f"1 M lattice: mixed vs FP64 p rel-L2 {res[1e-8]:.2e} at 1e-8, {res[1e-12]:.2e} at 1e-12")
    assert res[1e-8] <= 1e-6, res
    assert res[1e-12] <= 1e-7, res
