"""The oracle pinned to the reference itself: the reference's own scene run
through its own main program by the reference's Fortran source (translated
and compiled by oracle/ref_build.py, MKL's solve replaced by the reference's
own BiCGStab to a tight residual), against the oracle's restatement of the
same schedule (beachslope_gb300.aquifer: the scene generator and the
three-phase driver) with the PPE solved tightly by its BiCGStab.

Fixtures: tests/golden/ref_aquifer.npz, made by
tests/golden/make_ref_golden.py.  Particle order (cells column-major, slots
in order) is compared exactly; the set-up bit for bit; after steps the real
fields within the tolerances written in each assert (the two codes sum in
different orders; the fields' own step-to-step change is far larger).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ref_aquifer.npz")
REF_TREE = "/root/reference"


def _gold():
    return np.load(GOLD)


def _fix(g, name, k):
    pre = f"{name}_{k}_"
    return {key[len(pre):]: g[key] for key in g.files if key.startswith(pre)}


def relL2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


class _OracleCtx:
    """The oracle behind the Context calls run_schedule makes."""

    def __init__(self, o):
        self.o = o

    def prime(self):
        self.o.stage("prime")

    def prime_setup(self):
        self.o.stage("prime_setup")

    def step_flags(self, n, f):
        self.o.step_flags(n, f)

    def step(self, n=1):
        self.o.step(n)

    def download(self, s=0, full=True):
        return self.o.get()

    def set_fields(self, fields, s=0):
        self.o.set_fields(fields)

    def set_inflow(self, z, zd, s=0):
        self.o.set_inflow(z, zd)

    def set_time(self, t, s=0):
        self.o.set_time(t)

    def info(self, s=0):
        return self.o.info()


def tight_scene(periods=None):
    """The reference's scene with the PPE solved to rounding by BiCGStab, and
    the exchange periods of the fixture's short schedule."""
    from beachslope_gb300 import abi, aquifer as aq
    p, st, gr, zones, info = aq.aquifer_scene()
    p.ppe_solver = abi.SOLVER_BICGSTAB
    p.ppe_stop = abi.STOP_RELRES
    p.ppe_tol = 1e-13
    p.ppe_maxit = 20000
    if periods:
        for z, per in zip(zones, periods):
            z["period"] = per
    return p, st, gr, zones, info


def check_state(got, ref, exact=False, x_tol=1e-11, p_tol=1e-9, v_tol=1e-9, rho_tol=1e-12, con_tol=1e-12,
                mass_tol=1e-14):
    """got: a state in row order (cells column-major, slots in order); ref: a
    fixture dump.  Default bars: the oracle against the reference (measured
    in the build container after 10 steps of the three phases: positions
    1.3e-15 m, p 4e-13, vx 1e-12, rho 3.5e-16; after the 50 steps of the
    first phase: positions 1.4e-14 m, p 3.9e-13, v 5.3e-13, rho 2.6e-15)."""
    np.testing.assert_array_equal(got["tid"], ref["tid"])
    np.testing.assert_array_equal(got["flags"] & 4 != 0, ref["buffer"] != 0)   # BS_FLAG_BUFFER
    if exact:
        for f in ("x", "y", "vx", "vy", "p", "rho", "mass", "porosity"):
            np.testing.assert_array_equal(got[f], ref[f], err_msg=f)
        return {}
    dx = float(max(np.max(np.abs(got["x"] - ref["x"])), np.max(np.abs(got["y"] - ref["y"]))))
    e = {f: relL2(got[f], ref[f]) for f in ("p", "vx", "vy", "rho", "porosity", "con", "mass")}
    assert dx <= x_tol, (dx, e)
    assert e["p"] <= p_tol, e
    assert e["vx"] <= v_tol and e["vy"] <= v_tol, e
    assert e["rho"] <= rho_tol and e["porosity"] <= rho_tol, e
    assert e["con"] <= con_tol and e["mass"] <= mass_tol, e
    return dict(e, x=dx)


def test_oracle_setup_is_the_reference_setup(oracle):
    """init + gen_boundary + gen_fluid + memalloc + matrixid + effpor
    (main.f90:25-37) against aquifer_scene + prime: every particle in the
    same cell and slot, every field bit for bit."""
    p, st, gr, zones, info = tight_scene()
    o = oracle.Oracle(p, st, gr)
    o.stage("prime_setup")
    check_state(o.get(), _fix(_gold(), "all", 0), exact=True)


def test_oracle_schedule_matches_reference(oracle):
    """main.f90's three phases, cut to 3 + 3 + 4 steps with the buffers
    exchanging every 4.5 ms / 8.5 ms: the end of each phase."""
    from beachslope_gb300 import aquifer as aq
    p, st, gr, zones, info = tight_scene((0.0045, 0.0085))
    o = oracle.Oracle(p, st, gr)
    seen = {}

    def on_phase(name):
        seen[name] = (o.get(), o.info())

    aq.run_schedule(_OracleCtx(o), zones, info, settle1=3, settle2=3, production=4, on_phase=on_phase)
    g = _gold()
    for name, k in (("settled", 3), ("buffers_settled", 6), ("production", 10)):
        ref = _fix(g, "all", k)
        got, inf = seen[name]
        assert inf["t"] == pytest.approx(float(ref["t"]), abs=1e-15)
        e = check_state(got, ref)
        print(name, e)


def test_oracle_first_phase_matches_reference(oracle):
    """The first settling phase in full (50 steps, main.f90:39-64), with the
    adaptive time step (integrator.f90:885-953) taking the same values."""
    p, st, gr, zones, info = tight_scene()
    o = oracle.Oracle(p, st, gr)
    o.stage("prime_setup")
    o.step_flags(50, 0)
    ref = _fix(_gold(), "settle50", 50)
    assert o.info()["t"] == pytest.approx(float(ref["t"]), rel=1e-13)
    assert o.info()["dt"] == pytest.approx(float(ref["dt"]), rel=1e-13)
    e = check_state(o.get(), ref)
    print(e)


@pytest.mark.skipif(not os.path.isdir(REF_TREE), reason="the reference tree is only in the build container")
def test_fixture_is_what_the_reference_computes(tmp_path):
    """Rebuild the reference from its source and rerun the short schedule:
    the fixture's numbers, bit for bit."""
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import ref_build
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_ref_golden as mk
    exe = ref_build.build()
    pre = str(tmp_path / "all")
    subprocess.check_call([exe, pre, "3", "3", "4", "1000000", "0.0045", "0.0085"])
    g = _gold()
    for k in (0, 3, 6, 10):
        d = mk.load_dump(f"{pre}_{k}.bin")
        ref = _fix(g, "all", k)
        for f in ("x", "y", "vx", "vy", "p", "rho", "con", "porosity"):
            np.testing.assert_array_equal(d[f], ref[f], err_msg=f"{k} {f}")
