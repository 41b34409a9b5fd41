"""The reference's own scene and run schedule.

`aquifer_scene()` restates the reference's set-up -- `init` (setup.f90:10-150),
`gen_boundary` (boundary.f90:12-605) and `gen_fluid` (internal.f90:10-445) --
with the parameter defaults of initialize.f90:17-60: a coastal aquifer tank
with fixed and ghost wall layers, a fluid block spaced dx/sqrt(por) behind a
sloping coast line, a coastal water block above it, a porous soil lattice
below the line, an inflow buffer on the right and an open buffer at the
left.  Particles are listed in the reference's generation order, so the
upload's stable binning gives each cell the slot order of the reference's
lists (walls first, in wall-segment order; fluid blocks in their order), and
particles outside every interior cell are dropped as the reference's cell
loops drop them.  Wall and fluid pids count separately, as there.

`run_schedule()` is the three-phase driver of main.f90:39-272: 50 settling
steps without scalar transport, buffers, density update and the closing
eddyvis; the fluid velocities zeroed; the settling steps with the buffers
(insert_buffer2 at relative density 1); the salinity set-up (fluid above the
coast line denser, con = +0.5, the rest -0.5); t restarted at 0 with the
buffer schedule shifted by the elapsed time; the production steps, with the
`combined` output every `displaytime`.

The restatement is read from the reference's source; the reference itself
cannot be built here, so the scene is unpinned against a reference run.
"""
import math

import numpy as np

from . import abi, scene

# initialize.f90:17-60 (the values the generator reads)
DEFAULTS = dict(
    wc=0.650, L=3.11, H=0.80, pr=0.0050 * 0.90, br=0.00490 * 0.90, wl=3.10, rho=1000.0, g=-9.810,
    csh=0.50, rhomin=1000.0, tschmidt=1.0, soill=3.230, soilh=0.80, set_ht=0.20, coastal_ht=0.450,
    por=0.380, bulkden=1800.0, entry_vel=-2.5 / (3600 * 24), lhs_btm=0.20, rel_den=1.0250,
    dt=float(np.float32(0.001)),   # initialize.f90:32 writes 0.001 as a default (single precision) REAL
    time=7320.0, displaytime=100.0, mu=0.0010, sig1=0.20, maxshift=0.1,
    line_grad=16.690, lamfs=0.80, maxdivr=2.0, hfac=5.080, bl=3, open_lhs=43, incr=4,
)


def _geometry(c):
    """init, setup.f90:17-94 and 141-143 (the values of the module state)."""
    g = {}
    sq = math.sqrt(c["por"])
    fpy = math.floor(c["wc"] / (2 * c["pr"])) + 1
    fpx = math.floor(c["wl"] / (2 * c["pr"]))
    prx = (c["wl"] / fpx) / 2.0
    pry = (c["wc"] / (fpy - 1)) / 2.0
    g["fmass"] = ((c["wc"] * c["wl"] * 1.0) * c["rho"]) / (fpx * fpy)
    spy = math.floor(c["soilh"] / (2 * pry)) + 4
    spx = math.floor(c["soill"] / (2 * prx))
    g["solidx"] = (c["soill"] / spx) / 2.0
    g["solidy"] = (c["soilh"] / (spy - 1)) / 2.0
    L = c["L"]
    H = c["H"] + 2 * pry
    bny = math.floor(H / (2 * c["br"]))
    bnx = math.floor(L / (2 * c["br"]))
    brx = (L / bnx) / 2.0
    bry = (H / bny) / 2.0
    h1 = (max(prx, pry) * c["hfac"]) / (2.0 * sq)
    g["cellx"] = math.ceil(L / (c["incr"] * h1)) + 4
    g["celly"] = math.ceil(H / (c["incr"] * h1)) + 3
    g["dl"] = min(2 * prx, 2 * pry)
    bny = math.floor(c["lhs_btm"] / (2 * bry))
    bl = c["bl"]
    g["domain_shift"] = 5 * prx
    g["bnx"] = bnx + 2 * bl
    g["bny"] = bny + 2 * bl
    g["xl"] = (2 * bl - 1) * brx + brx
    g["yl"] = (2 * bl - 1) * bry + g["solidy"] + c["set_ht"]
    g["line_grad"] = (c["line_grad"] * 22) / (180.0 * 7)
    g["fpy"] = math.floor(c["wc"] / (2 * pry / sq))
    g["fpx"] = math.floor(c["wl"] / (2 * prx / sq))
    g["xrcutoff"] = (brx * ((2 * bl) - 1)) + (g["fpx"] - 1) * 2 * prx / sq + 3 * prx / sq + g["domain_shift"] - 0.001
    g["xlcutoff"] = (brx * ((2 * bl) - 1)) + brx
    g.update(prx=prx, pry=pry, spx=spx, spy=spy, brx=brx, bry=bry, h1=h1, L=L, H=H, sq=sq)
    return g


def _params(c, g, precision):
    """The run parameters the reference's modules hold after init."""
    p = abi.default_params()
    p.h = g["h1"]
    p.dl = g["dl"]
    p.cellx, p.celly = g["cellx"], g["celly"]
    p.dt = c["dt"]
    p.adaptive_dt = 1
    p.scalar_on = 1
    p.rho, p.rhomin, p.rel_den = c["rho"], c["rhomin"], c["rel_den"]
    p.rhomax = c["rho"] * c["rel_den"]   # setup.f90:19
    p.g, p.mu, p.tschmidt = c["g"], c["mu"], c["tschmidt"]
    p.por = c["por"]
    p.lamfs, p.maxdivr, p.csh, p.maxshift, p.sig1 = c["lamfs"], c["maxdivr"], c["csh"], c["maxshift"], c["sig1"]
    p.xlcutoff = g["xlcutoff"]
    # comp_pos releases buffer particles between these (integrator.f90:865-872)
    p.buf_release_lo = 8 * g["prx"] + g["brx"] + 0.001
    p.buf_release_hi = g["xrcutoff"]
    p.precision = precision
    # the reference's live solve (fgmres, solver.f90:306-350)
    p.ppe_solver = abi.SOLVER_FGMRES
    p.ppe_restart = 150
    p.ppe_maxit = 150
    p.ppe_stop = abi.STOP_R0
    p.ppe_tol = 1e-3
    p.ppe_precond = 0
    p.kmax = 64   # the coastal block is spaced 2 pr, denser than the porous blocks
    return p


def aquifer_scene(precision=abi.PREC_FP64, **overrides):
    """(params, state, grains, zones, info) of the reference's scene; zones =
    [buffer1 zone, buffer2 zone] dicts for Context.set_inflow (the buffer2
    zone at relative density 1, as the settling phase inserts it); info holds
    the scalars the driver needs."""
    c = dict(DEFAULTS)
    c.update(overrides)
    g = _geometry(c)
    p = _params(c, g, precision)
    bl, ds, brx, bry, prx, pry, sq = c["bl"], g["domain_shift"], g["brx"], g["bry"], g["prx"], g["pry"], g["sq"]
    fmass, rho, ag = g["fmass"], c["rho"], abs(c["g"])
    xs, ys, tids, pids, vxs, ps, masses, rhos, odens, ovols, flags = ([] for _ in range(11))

    def cell(x, y):
        return scene.cell_of(p, x, y)

    def add(x, y, tid, pid, vx=0.0, pr=0.0, mass=fmass, dens=rho, oden=0.0, ovol=0.0, buf=False):
        """Keep a particle that falls in an interior cell (the reference's
        binning loops run over cells 2..cellx-1, 2..celly-1)."""
        if cell(x, y) is None:
            return False
        xs.append(x); ys.append(y); tids.append(tid); pids.append(pid); vxs.append(vx); ps.append(pr)
        masses.append(mass); rhos.append(dens); odens.append(oden); ovols.append(ovol)
        flags.append(abi.FLAG_BUFFER if buf else 0)
        return True

    # ---- gen_boundary: the wall segments in order, binned column by column of
    # their lists (blist(k, m), k fastest)
    icount = 0
    bny = g["bny"]
    seg = {}
    for j in range(1, bl + 1):            # left wall below the open inlet
        for i in range(bny, 0, -1):
            tid = 1 if (j == bl and i <= bny - bl + 1) else 2
            icount += 1
            seg[(i, j)] = (tid, icount)
    for m in range(1, bl + 1):
        for k in range(1, bny + 1):
            tid, pid = seg[(k, m)]
            add((m - 1) * brx * 2 + ds, (bny - k) * bry * 2.0, tid, pid)
    remain = c["wc"] - c["lhs_btm"] - c["open_lhs"] * 2 * pry
    bn1 = math.floor(remain / (2 * bry)) - 2
    p.ytcutoff = (bny * 2 * bry) + (c["open_lhs"] * 2 * pry) + (bn1) * bry * 2 - bry   # boundary.f90:206
    seg = {}
    for j in range(1, bl + 1):            # left wall above the inlet
        for i in range(1, bn1 + 1):
            icount += 1
            seg[(i, j)] = (1 if j == bl else 2, icount)
    for m in range(1, bl + 1):
        for k in range(1, bn1 + 1):
            tid, pid = seg[(k, m)]
            add((m - 1) * brx * 2 + ds, (bny * 2 * bry) + (c["open_lhs"] * 2 * pry) + (bn1 - k) * bry * 2, tid, pid)
    nb = g["bnx"] - 2 * bl + 7
    seg = {}
    for j in range(1, nb + 1):            # bottom
        for i in range(1, bl + 1):
            icount += 1
            seg[(i, j)] = (1 if i == 1 else 2, icount)
    for m in range(1, nb + 1):
        for k in range(1, bl + 1):
            tid, pid = seg[(k, m)]
            add((2 * bl - 1) * brx + brx + (m - 1) * brx * 2 + ds, (bl - k) * 2 * bry, tid, pid)
    buy1 = g["fpy"] - 1
    seg = {}
    for j in range(1, bl + 1):            # upper right wall (20 rows)
        for i in range(1, 21):
            icount += 1
            seg[(i, j)] = (1 if j == 1 else 2, icount)
    for m in range(1, bl + 1):
        for k in range(1, 21):
            tid, pid = seg[(k, m)]
            y = ((bry * ((2 * bl) - 1)) + buy1 * 2 * pry / sq + 2 * pry / sq) + bry + (20 - k) * 2 * bry
            x = ((brx * ((2 * bl) - 1)) + (g["fpx"] - 1) * 2 * prx / sq + 3 * prx / sq) + (m - 1) * 2 * brx + ds
            add(x, y, tid, pid)
    # porous soil lattice (porlist): below the coast line only
    gx, gy = [], []
    spx, spy, sx, sy = g["spx"], g["spy"], g["solidx"], g["solidy"]
    gmass = c["soill"] * c["soilh"] * c["bulkden"] / (spx * spy)
    xl, yl, lg = g["xl"], g["yl"], g["line_grad"]
    for l1 in range(1, spx + 1):
        for k in range(1, spy + 1):
            y = (spy - k) * 2 * sy + sy + (bry * ((2 * bl) - 1)) - 6 * sy
            x = (brx * ((2 * bl) - 1)) + (l1 - 1) * 2 * sx + brx - 6 * sx + ds
            if ((y - yl) - lg * (x - xl)) > 0.0:
                continue
            if cell(x, y) is not None:
                gx.append(x); gy.append(y)
    grains = {"x": np.array(gx), "y": np.array(gy), "mass": np.full(len(gx), gmass),
              "rho": np.full(len(gx), c["bulkden"])}

    # ---- gen_fluid
    fpy, fpx = g["fpy"], g["fpx"]
    base_x, base_y = brx * ((2 * bl) - 1), bry * ((2 * bl) - 1)
    bounlen, bounlen2 = fpy * 2 * pry, c["open_lhs"] * 2 * pry
    ins_1 = (4 * prx / sq) / abs(c["entry_vel"] / 0.387)
    ins_2 = 4 * prx / ((bounlen / bounlen2) * abs(c["entry_vel"]))
    rv_buf_r = base_x + (fpx - 1) * 2 * prx / sq + prx / sq + ds + 3 * 2 * prx / sq + 0.5 * prx / sq
    rv_buf_l = 2 * prx + brx + 0.5 * prx
    wlev_p = lambda y: (-y + base_y + c["wc"] + pry / sq) * rho * ag   # noqa: E731
    count = 0
    pid_of = {}
    for j in range(1, fpx + 1):            # main block: pids bottom to top
        for i in range(fpy, 0, -1):
            count += 1
            pid_of[(i, j)] = count
    for l1 in range(1, fpx + 1):
        for k in range(1, fpy + 1):
            y = base_y + (fpy - k) * 2 * pry / sq + pry / sq
            x = base_x + (l1 - 1) * 2 * prx / sq + prx / sq + ds
            if ((y - yl) - lg * (x - xl)) > 0.0:
                continue
            add(x, y, 3, pid_of[(k, l1)], vx=c["entry_vel"], pr=wlev_p(y), oden=rho, ovol=fmass / rho)
    # right buffer: 5 columns, the last 2 are the template buffer1
    entry1 = []
    pid_of = {}
    for j in range(1, 6):
        for i in range(fpy, 0, -1):
            count += 1
            pid_of[(i, j)] = count
    t1 = {"x": [], "y": [], "p": []}
    for l1 in range(1, 6):
        for k in range(1, fpy + 1):
            y = base_y + (fpy - k) * 2 * pry / sq + pry / sq
            x = base_x + (fpx - 1) * 2 * prx / sq + prx / sq + ds + l1 * 2 * prx / sq
            if add(x, y, 3, pid_of[(k, l1)], vx=c["entry_vel"], pr=wlev_p(y), oden=rho, ovol=fmass / rho, buf=True):
                cc = cell(x, y)
                if cc not in entry1:
                    entry1.append(cc)
    for col in (4, 5):                     # insert order: template column, then row from the top
        for k in range(1, fpy + 1):
            y = base_y + (fpy - k) * 2 * pry / sq + pry / sq
            t1["x"].append(base_x + (fpx - 1) * 2 * prx / sq + prx / sq + ds + col * 2 * prx / sq)
            t1["y"].append(y)
            t1["p"].append(wlev_p(y))
    entry1.sort(key=lambda c_: (c_[1], c_[0]))
    # coastal block above the line (spacing 2 pr), pressures to coastal_ht
    fpy2 = math.floor(c["coastal_ht"] / (2 * pry)) + 1
    fpx2 = math.floor(2.0 / (2 * prx))
    dl = g["dl"]
    pid_of = {}
    for j in range(1, fpx2 + 1):
        for i in range(fpy2, 0, -1):
            count += 1
            pid_of[(i, j)] = count
    for l1 in range(1, fpx2 + 1):
        for k in range(1, fpy2 + 1):
            y = base_y + (fpy2 - k) * 2 * pry + pry + c["set_ht"]
            x = base_x + (l1 - 1) * 2 * prx + prx + ds
            pr = 0.0 if k == 1 else (-y + (bry * ((2 * bl) - 1)) + c["coastal_ht"] + pry + c["set_ht"]) * rho * ag
            if ((y - yl + pry) - lg * (x - xl)) < 0.0:
                continue
            add(x, y + 2 * dl, 3, pid_of[(k, l1)], pr=pr, oden=rho, ovol=fmass / rho)
    # left open buffer: 5 columns, the first 2 are the template buffer2
    olhs = c["open_lhs"]
    bnyv = g["bny"]
    vx2 = (-bounlen / bounlen2) * c["entry_vel"]
    pid_of = {}
    for j in range(1, 6):
        for i in range(1, olhs + 1):
            count += 1
            pid_of[(i, j)] = count
    entry2 = []
    t2 = {"x": [], "y": [], "p": []}
    lhs_p = lambda y: (-y + base_y + c["wc"] + pry) * rho * ag   # noqa: E731
    for l1 in range(1, 6):
        for k in range(1, olhs + 1):
            y = 2 * bnyv * bry - bry + pry + (olhs - k) * 2 * pry
            x = (l1 - 1) * 2 * prx + brx
            if add(x, y, 3, pid_of[(k, l1)], vx=vx2, pr=lhs_p(y), oden=rho, ovol=fmass / rho, buf=True):
                cc = cell(x, y)
                if cc[1] <= g["cellx"] // 2 and cc not in entry2:
                    entry2.append(cc)
    for col in (1, 2):
        for k in range(1, olhs + 1):
            y = 2 * bnyv * bry - bry + pry + (olhs - k) * 2 * pry
            t2["x"].append((col - 1) * 2 * prx + brx)
            t2["y"].append(y)
            t2["p"].append(lhs_p(y) * c["rel_den"])
    entry2.sort(key=lambda c_: (c_[1], c_[0]))

    n = len(xs)
    st = {"x": np.array(xs), "y": np.array(ys), "vx": np.array(vxs), "vy": np.zeros(n), "p": np.array(ps),
          "mass": np.array(masses), "rho": np.array(rhos), "oden": np.array(odens), "ovol": np.array(ovols),
          "con": np.zeros(n), "tid": np.array(tids, np.int32), "pid": np.array(pids, np.int32),
          "flags": np.array(flags, np.uint8)}

    def zone(t, cells, mass, dens, con, period, remove_x, side, vx):
        m = len(t["x"])
        return {"x": np.array(t["x"]), "y": np.array(t["y"]), "vx": np.full(m, vx), "vy": np.zeros(m),
                "p": np.array(t["p"]), "pid": None, "mass": mass, "rho": dens, "ovol": fmass / rho, "con": con,
                "period": period, "phase": 0.0, "remove_x": remove_x, "remove_side": side, "cells": cells}

    zones = [zone(t1, entry1, fmass, rho, -0.5, ins_1, rv_buf_r, 1, c["entry_vel"]),
             zone(t2, entry2, fmass, rho, 0.5, ins_2, rv_buf_l, -1, vx2)]
    info = {"fmass": fmass, "rel_den": c["rel_den"], "xl": xl, "yl": yl, "line_grad": lg,
            "time": c["time"], "displaytime": c["displaytime"], "ins_1": ins_1, "ins_2": ins_2}
    return p, st, grains, zones, info


# the largest step the reference's time-step rule takes (integrator.f90:927-936)
DT_MAX = 0.005


def salinity_setup(state, info):
    """main.f90:156-191: every fluid particle con = -0.5; fluid above the
    coast line denser by rel_den (mass, oden, density) and con = +0.5.
    Returns the fields for set_fields."""
    fl = state["tid"] == abi.TID_FLUID
    above = fl & (((state["y"] - info["yl"]) - info["line_grad"] * (state["x"] - info["xl"])) > 0.0)
    rd = info["rel_den"]
    return {"mass": np.where(above, state["mass"] * rd, state["mass"]),
            "oden": np.where(above, state["oden"] * rd, state["oden"]),
            "rho": np.where(above, state["rho"] * rd, state["rho"]),
            "con": np.where(fl, np.where(above, 0.5, -0.5), state["con"])}


def run_schedule(ctx, zones, info, settle1=50, settle2=8000, production=None, out_dir=None, s=0, on_phase=None):
    """main.f90:39-272 on scene s of a Context made from aquifer_scene()
    (before prime).  production=None runs until the reference's end time
    (`time`); otherwise that many production steps.  With out_dir, the
    combined output goes to out_dir/fluid/fluid_<1000+k>.txt and
    out_dir/buffer/buffer_<1000+k>.txt: k = 0 before the first step, one file
    pair per `displaytime` of production, and a last pair at the end
    (output.f90:186-223).  on_phase(name) runs after each part: "settled",
    "at_rest", "buffers_settled", "salted", "production".  Returns the
    number of production steps."""
    import os

    def dump(k):
        if out_dir is not None:
            os.makedirs(os.path.join(out_dir, "fluid"), exist_ok=True)
            os.makedirs(os.path.join(out_dir, "buffer"), exist_ok=True)
            ctx.write_combined(os.path.join(out_dir, "fluid", f"fluid_{1000 + k}.txt"),
                               os.path.join(out_dir, "buffer", f"buffer_{1000 + k}.txt"), s=s)

    def phase(name):
        if on_phase is not None:
            on_phase(name)

    dump(0)
    ctx.prime_setup()   # main.f90:23-37: no time-step rule before the first step
    # settling without buffers, scalar transport, density update or the
    # closing eddyvis (main.f90:39-67); then the fluid at rest
    ctx.step_flags(settle1, 0)
    phase("settled")
    st = ctx.download(s, full=False)
    still = (st["tid"] == abi.TID_FLUID) & ((st["flags"] & abi.FLAG_BUFFER) == 0)
    ctx.set_fields({"vx": np.where(still, 0.0, st["vx"]), "vy": np.where(still, 0.0, st["vy"])}, s)
    phase("at_rest")
    # settling with the buffers, the open side at relative density 1
    # (main.f90:95-147; the exchange counters start again at 1)
    for z, zd in enumerate(zones):
        ctx.set_inflow(z, zd, s)
    ctx.step_flags(settle2, abi.STEP_BUFFERS)
    phase("buffers_settled")
    # salt water above the coast line, t from 0 with the buffer schedule
    # shifted by the settling time (main.f90:149-197)
    st = ctx.download(s, full=False)
    ctx.set_fields(salinity_setup(st, info), s)
    t_shift = ctx.info(s)["t"]
    ctx.set_time(0.0, s)
    for z, zd in enumerate(zones):
        zd = dict(zd, phase=t_shift)
        if z == 1:
            zd["mass"] = info["fmass"] * info["rel_den"]
            zd["rho"] = zones[1]["rho"] * info["rel_den"]
        ctx.set_inflow(z, zd, s)
    phase("salted")
    # steps run in chunks that cannot reach the next output time or the end:
    # the time-step rule never takes dt above DT_MAX, so n steps with
    # n DT_MAX <= (target - t) stay short of it, and the step that crosses a
    # target is taken alone (the outputs fall on the same steps as one step
    # at a time, with one host read of t per chunk)
    steps, k = 0, 1
    t = ctx.info(s)["t"]
    while (t < info["time"]) if production is None else (steps < production):
        target = k * info["displaytime"]
        if production is None:
            target = min(target, info["time"])
        n = max(1, int((target - t) / DT_MAX))
        if production is not None:
            n = min(n, production - steps)
        told = t
        ctx.step(n)
        steps += n
        t = ctx.info(s)["t"]
        if told < k * info["displaytime"] <= t:
            dump(k)
            k += 1
    phase("production")
    dump(k)
    return steps
