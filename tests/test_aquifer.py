"""The reference's own scene (init + gen_boundary + gen_fluid: setup.f90,
boundary.f90, internal.f90) and its three-phase run (main.f90:39-272).

The reference cannot be built here (no Fortran compiler), so the scene is
not pinned against a run of it: the CPU tests check the generator against
the facts its loops imply (segment sizes, pid order, the coast line, the
buffer templates lying on the buffer columns, the entry cells), and the
driver on the oracle; the GPU tests run the same short schedule on the
library and on the oracle and compare every phase.
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def aq():
    from beachslope_gb300 import aquifer
    return aquifer


def _short(aq, periods=(0.0045, 0.0085), **kw):
    """The scene with exchanges every few steps.  The schedule counts
    exchanges from k = 1 in each phase and fires when (t_old + phase) <
    k period <= (t + phase), so with 3 + 3 settling steps of 1 ms buffer1
    (4.5 ms) exchanges in the second settling phase only and buffer2
    (8.5 ms, phase 6 ms in production) in the production steps only."""
    p, st, gr, zones, info = aq.aquifer_scene(**kw)
    for z, per in zip(zones, periods):
        z["period"] = per
    return p, st, gr, zones, info


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

    def write_combined(self, f, b=None, s=0):
        self.o.write_combined(f, b)


def test_generator_layout(aq):
    from beachslope_gb300 import abi, scene
    p, st, gr, zones, info = aq.aquifer_scene()
    n = len(st["x"])
    wall = st["tid"] <= 2
    fl = st["tid"] == abi.TID_FLUID
    buf = (st["flags"] & abi.FLAG_BUFFER) > 0
    assert n == wall.sum() + fl.sum() and wall.sum() > 1000 and fl.sum() > 10000
    # every particle lies in an interior cell; walls come first in the list
    assert all(scene.cell_of(p, x, y) is not None for x, y in zip(st["x"], st["y"]))
    assert np.all(np.diff(wall.astype(int)) <= 0)
    # pids: walls and fluid each unique
    assert len(np.unique(st["pid"][wall])) == wall.sum()
    assert len(np.unique(st["pid"][fl])) == fl.sum()
    # buffers: 5 columns of fpy (right) and of open_lhs (left) particles
    d = aq.DEFAULTS
    right = buf & (st["x"] > 1.0)
    assert right.sum() == 5 * len(zones[0]["x"]) // 2
    assert (buf & ~right).sum() == 5 * d["open_lhs"] == 5 * len(zones[1]["x"]) // 2
    # no two particles at one place
    xy = np.round(np.c_[st["x"], st["y"]] / 1e-9).astype(np.int64)
    assert len(np.unique(xy, axis=0)) == n
    # the porous block and the grains lie below the coast line, the coastal
    # block above it
    line = lambda x, y: (y - info["yl"]) - info["line_grad"] * (x - info["xl"])   # noqa: E731
    assert np.all(line(gr["x"], gr["y"]) <= 0.0)
    main = fl & ~buf & (np.abs(st["vx"] - d["entry_vel"]) == 0)
    coast = fl & ~buf & (st["vx"] == 0.0)
    assert main.sum() + coast.sum() == (fl & ~buf).sum()
    assert np.all(line(st["x"][main], st["y"][main]) <= 0.0)
    assert np.all(line(st["x"][coast], st["y"][coast]) > 0.0)
    # the free surface rows of the coastal block start at p = 0
    assert np.any(coast & (st["p"] == 0.0)) and np.all(st["p"][fl] >= 0.0)


def test_generator_zones(aq):
    from beachslope_gb300 import abi, scene
    p, st, gr, zones, info = aq.aquifer_scene()
    buf = (st["flags"] & abi.FLAG_BUFFER) > 0
    pos = {(x, y) for x, y in zip(st["x"][buf], st["y"][buf])}
    for z, zd in enumerate(zones):
        # the template is the buffer's outer two columns, column by column,
        # top row first (insert_buffer1/2)
        assert all((x, y) in pos for x, y in zip(zd["x"], zd["y"]))
        m = len(zd["x"]) // 2
        for half in (slice(0, m), slice(m, 2 * m)):
            assert len(np.unique(zd["x"][half])) == 1
            assert np.all(np.diff(zd["y"][half]) < 0)
        # entry cells: every cell that holds a particle of the zone, ordered
        # by column then row
        side = (st["x"] > 1.0) if z == 0 else (st["x"] < 1.0)
        cells = {scene.cell_of(p, x, y) for x, y in zip(st["x"][buf & side], st["y"][buf & side])}
        assert set(map(tuple, zd["cells"])) == cells
        assert list(zd["cells"]) == sorted(zd["cells"], key=lambda c: (c[1], c[0]))
        assert all((j > p.cellx // 2) == (z == 0) for _, j in zd["cells"])
    # an exchange removes the buffer particles still on the template's
    # columns: buffer1 at or right of rv_buf_r, a quarter spacing left of
    # the template; buffer2 at or left of rv_buf_l, a quarter spacing right
    z0, z1 = zones
    sp0 = np.ptp(z0["x"])
    assert z0["remove_side"] == 1 and z0["x"].min() - sp0 < z0["remove_x"] < z0["x"].min()
    sp1 = np.ptp(z1["x"])
    assert z1["remove_side"] == -1 and z1["x"].max() < z1["remove_x"] < z1["x"].max() + sp1
    # the open side's template pressures carry rel_den, buffer1's do not
    rows = {(x, y): q for q, (x, y) in enumerate(zip(st["x"], st["y"]))}
    q1 = [rows[(x, y)] for x, y in zip(z1["x"], z1["y"])]
    np.testing.assert_array_equal(z1["p"], st["p"][q1] * info["rel_den"])
    q0 = [rows[(x, y)] for x, y in zip(z0["x"], z0["y"])]
    np.testing.assert_array_equal(z0["p"], st["p"][q0])
    assert z0["con"] == -0.5 and z1["con"] == 0.5
    # the release window of comp_pos lies between the two zones
    assert z1["x"].max() < p.buf_release_lo < p.buf_release_hi < z0["x"].min()


def test_schedule_oracle(aq, oracle):
    """The three phases on the oracle with exchanges made frequent: what each
    hand-off between phases changes."""
    from beachslope_gb300 import abi
    p, st, gr, zones, info = _short(aq)
    o = oracle.Oracle(p, st, gr)
    seen = {}

    def on_phase(name):
        seen[name] = (o.get(), o.info())

    steps = aq.run_schedule(_OracleCtx(o), zones, info, settle1=3, settle2=3, production=4, on_phase=on_phase)
    assert steps == 4 and list(seen) == ["settled", "at_rest", "buffers_settled", "salted", "production"]
    g, _ = seen["at_rest"]
    still = (g["tid"] == 3) & ((g["flags"] & abi.FLAG_BUFFER) == 0)
    assert np.all(g["vx"][still] == 0.0) and np.all(g["vy"][still] == 0.0)
    assert np.any(g["vx"][~still & (g["tid"] == 3)] != 0.0)
    g0, _ = seen["buffers_settled"]
    new = (g0["pid"] == 0) & (g0["tid"] == 3)
    assert new.any() and np.all(g0["x"][new] > 1.0)
    assert np.all(g0["mass"][new] == info["fmass"]) and np.all(g0["con"][new] == -0.5)
    g, inf = seen["salted"]
    fl = g["tid"] == 3
    up = fl & (g["con"] == 0.5)
    assert up.sum() > 1000 and np.all(g["con"][fl & ~up] == -0.5)
    np.testing.assert_array_equal(g["mass"][up], g0["mass"][up] * info["rel_den"])
    np.testing.assert_array_equal(g["mass"][fl & ~up], g0["mass"][fl & ~up])
    assert inf["t"] == 0.0
    g, inf = seen["production"]
    assert inf["t"] == pytest.approx(4 * p.dt) and inf["err_bits"] == 0
    # buffer2's exchange in production inserts salt water (rel_den, con +0.5)
    left = (g["pid"] == 0) & (g["tid"] == 3) & (g["x"] < 1.0)
    assert left.sum() == len(zones[1]["x"])
    assert np.all(g["mass"][left] == info["fmass"] * info["rel_den"]) and np.all(g["con"][left] == 0.5)


def test_outputs_oracle(aq, oracle, tmp_path):
    p, st, gr, zones, info = _short(aq)
    info = dict(info, displaytime=0.0015)
    o = oracle.Oracle(p, st, gr)
    aq.run_schedule(_OracleCtx(o), zones, info, settle1=1, settle2=1, production=4, out_dir=str(tmp_path))
    names = sorted(f.name for f in (tmp_path / "fluid").iterdir())
    assert names == ["fluid_1000.txt", "fluid_1001.txt", "fluid_1002.txt", "fluid_1003.txt"]
    assert len((tmp_path / "buffer" / "buffer_1003.txt").read_text().splitlines()) > 300


def _compare(g, r, what, tol_x=1e-11, tol_p=1e-8):
    np.testing.assert_array_equal(g["pid"], r["pid"], err_msg=what)
    np.testing.assert_array_equal(g["flags"], r["flags"], err_msg=what)
    # salinity: exact through the hand-offs; the scalar transport's
    # neighbour sums then differ in the last bit
    assert np.max(np.abs(g["con"] - r["con"])) < 1e-12, what
    np.testing.assert_array_equal(g["mass"], r["mass"], err_msg=what)
    assert np.max(np.abs(g["x"] - r["x"])) < tol_x, what
    assert np.max(np.abs(g["y"] - r["y"])) < tol_x, what
    assert np.linalg.norm(g["p"] - r["p"]) / np.linalg.norm(r["p"]) < tol_p, what


@pytest.mark.gpu
def test_schedule_gpu_matches_oracle(api, aq, oracle):
    """The short schedule with a tight pressure solve on both sides: every
    phase hand-off agrees (positions 1e-11, pressure rel-L2 1e-8, salinity
    1e-12; ids, flags and masses exact)."""
    from beachslope_gb300 import abi
    p, st, gr, zones, info = _short(aq)
    p.ppe_solver, p.ppe_stop, p.ppe_tol, p.ppe_maxit, p.ppe_precond = abi.SOLVER_BICGSTAB, abi.STOP_RELRES, \
        1e-12, 20000, 1
    ctx = api.Context([p], [st], [gr], capacity=[len(st["x"]) + 1024])
    o = oracle.Oracle(p, st, gr)
    got, want = {}, {}
    aq.run_schedule(ctx, zones, info, settle1=3, settle2=3, production=4,
                    on_phase=lambda n: got.__setitem__(n, (ctx.download(), ctx.info())))
    aq.run_schedule(_OracleCtx(o), zones, info, settle1=3, settle2=3, production=4,
                    on_phase=lambda n: want.__setitem__(n, (o.get(), o.info())))
    for name in want:
        (g, gi), (r, ri) = got[name], want[name]
        _compare(g, r, name)
        assert gi["t"] == ri["t"] and gi["dt"] == ri["dt"], name
        assert gi["err_bits"] == 0, name
    assert np.any(got["production"][0]["pid"] == 0)


@pytest.mark.gpu
def test_reference_solver_gpu_matches_oracle(api, aq, oracle):
    """The reference's own solve (FGMRES, restart 150, |r| <= 1e-3 |r0|, no
    preconditioner) through the schedule: the same iteration counts and
    pressures to 1e-6."""
    p, st, gr, zones, info = _short(aq)
    ctx = api.Context([p], [st], [gr], capacity=[len(st["x"]) + 1024])
    o = oracle.Oracle(p, st, gr)
    got, want = {}, {}
    aq.run_schedule(ctx, zones, info, settle1=2, settle2=2, production=3,
                    on_phase=lambda n: got.__setitem__(n, (ctx.download(), ctx.info())))
    aq.run_schedule(_OracleCtx(o), zones, info, settle1=2, settle2=2, production=3,
                    on_phase=lambda n: want.__setitem__(n, (o.get(), o.info())))
    for name in want:
        (g, gi), (r, ri) = got[name], want[name]
        _compare(g, r, name, tol_x=1e-9, tol_p=1e-6)
        assert abs(gi["ppe_iters"] - ri["ppe_iters"]) <= 1, name
        assert gi["err_bits"] == 0, name


def test_reference_scene_size(aq):
    """The scene the reference's defaults give (initialize.f90:21-60): a
    46 x 14 cell grid, h1 = 18.6 mm, 1,233 wall and 12,448 fluid particles
    (435 in the two buffers), 25,643 soil grains, 88 + 86 template particles."""
    from beachslope_gb300 import abi
    p, st, gr, zones, info = aq.aquifer_scene()
    assert (p.cellx, p.celly) == (46, 14)
    assert abs(p.h - 0.0185991365) < 1e-9
    assert (st["tid"] <= 2).sum() == 1233 and (st["tid"] == abi.TID_FLUID).sum() == 12448
    assert ((st["flags"] & abi.FLAG_BUFFER) > 0).sum() == 435
    assert len(gr["x"]) == 25643
    assert [len(z["x"]) for z in zones] == [88, 86]


def test_production_chunks_keep_output_steps(aq, oracle, tmp_path):
    """Production runs in chunks of steps that cannot reach the next output
    time; the outputs land on the same steps as one step at a time (the same
    files, byte for byte; the oracle on one thread, whose sums are then in a
    fixed order)."""
    import os
    oracle.set_threads(1)
    try:
        _chunks_vs_single(aq, oracle, tmp_path)
    finally:
        oracle.set_threads(os.cpu_count() or 1)


def _chunks_vs_single(aq, oracle, tmp_path):
    p, st, gr, zones, info = _short(aq, periods=(1.0, 1.0))
    info = dict(info, displaytime=0.012)
    a = tmp_path / "chunked"
    o = oracle.Oracle(p, st, gr)
    aq.run_schedule(_OracleCtx(o), zones, info, settle1=1, settle2=1, production=30, out_dir=str(a))

    class OneByOne(_OracleCtx):
        def step(self, n=1):
            for _ in range(n):
                self.o.step(1)
            self.calls = getattr(self, "calls", 0) + n

    b = tmp_path / "single"
    ob = OneByOne(oracle.Oracle(p, st, gr))
    aq.run_schedule(ob, zones, info, settle1=1, settle2=1, production=30, out_dir=str(b))
    names = sorted(f.name for f in (a / "fluid").iterdir())
    assert names == sorted(f.name for f in (b / "fluid").iterdir())
    assert names == ["fluid_1000.txt", "fluid_1001.txt", "fluid_1002.txt", "fluid_1003.txt"]
    for n in names:
        assert (a / "fluid" / n).read_bytes() == (b / "fluid" / n).read_bytes(), n


def test_reference_scene_bytes(aq):
    """Regression pin of the generated scene: SHA-1 over the particles' x,
    y, p, vx, mass, tid, pid, flags, the grains' x, y and both zones'
    templates and entry cells (IEEE arithmetic in the reference's operation
    order, so the bytes are the same on every platform)."""
    import hashlib
    p, st, gr, zones, info = aq.aquifer_scene()
    h = hashlib.sha1()
    for k in ("x", "y", "p", "vx", "mass"):
        h.update(np.ascontiguousarray(st[k]).tobytes())
    h.update(st["tid"].tobytes())
    h.update(st["pid"].tobytes())
    h.update(st["flags"].tobytes())
    for k in ("x", "y"):
        h.update(gr[k].tobytes())
    for z in zones:
        h.update(z["x"].tobytes())
        h.update(z["y"].tobytes())
        h.update(z["p"].tobytes())
        h.update(np.asarray(z["cells"], np.int32).tobytes())
    assert h.hexdigest() == "9a24ea2262d527380aa3a2fec5920ba942508ae3"
