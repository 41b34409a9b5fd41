"""Synthetic scenes of the named shapes.

The reference only generates its own aquifer tank (boundary.f90:12-605,
internal.f90:10-445); the beach-slope scenes here are new and seeded.  Walls
follow the reference's convention: three layers (bl=3, initialize.f90:58),
the layer touching the fluid is tid=1 (fixed), the outer layers tid=2
(ghost); fluid is tid=3; grains of the porous bed are separate static
particles (porlist, boundary.f90:582-585) with mass/density = one lattice
cell of volume.  Cell geometry follows setup.f90:51-52,120-123: cells of
width 4h, x from 0 in column 2, an empty border ring.
"""
import math

import numpy as np

from . import abi


def _grid_for(p, xmax, ymax):
    cw = 4.0 * p.h
    p.cellx = int(math.ceil(xmax / cw)) + 3
    p.celly = int(math.ceil(ymax / cw)) + 3


def _mk(xs, ys, tid, mass, rho, oden, ovol, con, vx=None, vy=None, p=None):
    n = len(xs)
    z = np.zeros(n)
    return {
        "x": np.asarray(xs, float), "y": np.asarray(ys, float),
        "vx": z.copy() if vx is None else np.asarray(vx, float),
        "vy": z.copy() if vy is None else np.asarray(vy, float),
        "p": z.copy() if p is None else np.asarray(p, float),
        "mass": np.full(n, mass) if np.isscalar(mass) else np.asarray(mass, float),
        "rho": np.full(n, rho) if np.isscalar(rho) else np.asarray(rho, float),
        "oden": np.full(n, oden) if np.isscalar(oden) else np.asarray(oden, float),
        "ovol": np.full(n, ovol) if np.isscalar(ovol) else np.asarray(ovol, float),
        "con": np.full(n, con) if np.isscalar(con) else np.asarray(con, float),
        "tid": np.asarray(tid, np.int32),
    }


def _cat(parts):
    out = {}
    for k in parts[0]:
        out[k] = np.concatenate([q[k] for q in parts])
    out["pid"] = np.arange(1, len(out["x"]) + 1, dtype=np.int32)
    out["flags"] = np.zeros(len(out["x"]), np.uint8)
    return out


def _wab(r, h):
    """Hybrid kernel value (kernel.f90:34-66), vectorised."""
    q = r / h
    c28 = float(np.float32(28.0) * np.float32(3.14))
    c3 = float(np.float32(3.0) * np.float32(3.14))
    t1 = np.where(q < 1, 4.0 - 6.0 * q * q + 3.0 * q ** 3, (2.0 - q) ** 3)
    t2 = np.where(q < 1, q ** 3 - 6.0 * q + 6.0, (2.0 - q) ** 3)
    return 0.1 * t1 * (10.0 / (c28 * h * h)) + 0.9 * t2 * (1.0 / (c3 * h * h))


def porosity_field(x, y, grains, h, por):
    """phi = 1 - min(sum (1-por) W V_s, 1-por) over grains within 2h
    (porsearch/effpor, porous.f90:32-190), for scene set-up."""
    phi = np.ones(len(x))
    if len(grains["x"]) == 0 or len(x) == 0:
        return phi
    from scipy.spatial import cKDTree
    tg = cKDTree(np.c_[grains["x"], grains["y"]])
    tf = cKDTree(np.c_[x, y])
    pairs = tf.sparse_distance_matrix(tg, 2.0 * h, output_type="ndarray")
    vol = grains["mass"] / grains["rho"]
    fi, gi = pairs["i"], pairs["j"]
    r = np.hypot(x[fi] - grains["x"][gi], y[fi] - grains["y"][gi])
    m = r < 2.0 * h
    sf = np.bincount(fi[m], weights=(1.0 - por) * _wab(r[m], h) * vol[gi[m]], minlength=len(x))
    return 1.0 - np.minimum(sf, 1.0 - por)


def beach_scene(dx=0.01, L=4.0, H=0.6, depth=0.30, slope=0.1, toe=2.0, thick=0.05,
                por=0.40, d50=0.005, A=0.06, x0=None, layers=3, saline_beach=True,
                hfac=1.3, dt=1e-4, ppe_tol=1e-8, precision=abi.PREC_FP64, wcsph=False):
    """Solitary wave on a porous beach slope in a 2-D tank.

    Tank [0,L]x[0,H] (inner), still depth `depth`, impermeable slope of
    gradient `slope` from x=`toe`, a porous grain layer `thick` (normal to the
    slope) on it.  First-order Boussinesq solitary wave
    eta = A sech^2(k(x-x0)), k = sqrt(3A/(4 d^3)), u = sqrt(g/d) eta.
    The crest sits at x0 (default toe/2: a 4 m tank cannot hold the crest
    3/k upstream of a toe at 2 m).
    With wcsph=True the state is set up for the WCSPH step: every fluid
    particle carries the full lattice mass rho0*dx^2 (the grains still set
    porosity and drag) and the hydrostatic Tait density of its depth; the
    speed of sound is 10 sqrt(g d) and the still-water level d.
    Returns (params, state dict, grains dict).
    """
    p = abi.default_params()
    p.h = hfac * dx
    p.dl = dx
    p.dt = dt
    p.por = por
    p.d50 = d50
    p.ppe_tol = ppe_tol
    p.precision = precision
    rho, g = p.rho, p.g
    X0 = Y0 = (layers + 0.5) * dx
    d = depth
    k = math.sqrt(3.0 * A / (4.0 * d ** 3)) if A > 0 else 0.0
    if x0 is None:
        x0 = 0.5 * toe
    c0 = math.sqrt(-g / d)
    nx = int(round(L / dx))
    ny = int(round(H / dx))
    xs = X0 + (np.arange(nx) + 0.5) * dx

    def eta(x):
        if A <= 0:
            return np.zeros_like(x)
        return A / np.cosh(k * (x - X0 - x0)) ** 2

    def yslope(x):   # slope surface height above the tank floor
        return np.maximum(0.0, slope * (x - X0 - toe))

    parts = []
    fmass = rho * dx * dx
    # the right wall stands one spacing beyond the last fluid column (at
    # X0 + nx dx, which is L when L/dx is an integer): a wall closer than
    # dx to the fluid lattice, or further, makes the wall pressure blow up
    Lw = nx * dx
    # --- walls: bottom (full width incl. corners), left, right
    wx, wy, wt = [], [], []
    for lay in range(layers):
        tid = abi.TID_WALL if lay == 0 else abi.TID_GHOST
        xb = X0 + (np.arange(-layers, nx + layers) + 0.5) * dx
        yb = np.full_like(xb, Y0 - (lay + 0.5) * dx)
        tb = np.where((xb > X0) & (xb < X0 + Lw), tid, abi.TID_GHOST)
        wx.append(xb); wy.append(yb); wt.append(tb)
        yl = Y0 + (np.arange(ny) + 0.5) * dx
        wx.append(np.full_like(yl, X0 - (lay + 0.5) * dx)); wy.append(yl); wt.append(np.full(ny, tid))
        wx.append(np.full_like(yl, X0 + Lw + (lay + 0.5) * dx)); wy.append(yl); wt.append(np.full(ny, tid))
    # --- slope wall: lattice points within `layers` spacings below the slope surface
    gx, gy = np.meshgrid(xs, Y0 + (np.arange(ny) + 0.5) * dx, indexing="ij")
    gx = gx.ravel(); gy = gy.ravel()
    ysl = yslope(gx)
    below = (gy - Y0 < ysl) & (gy - Y0 >= ysl - layers * dx) & (gx - X0 > toe)
    depth_in = np.floor((ysl - (gy - Y0)) / dx)
    wx.append(gx[below]); wy.append(gy[below])
    wt.append(np.where(depth_in[below] < 1, abi.TID_WALL, abi.TID_GHOST))
    wx = np.concatenate(wx); wy = np.concatenate(wy); wt = np.concatenate(wt)
    pw = rho * (-g) * np.maximum(0.0, d - (wy - Y0))
    parts.append(_mk(wx, wy, wt, fmass, rho, 0.0, 0.0, 0.0, p=pw))
    # --- fluid
    fl = (gy - Y0 >= ysl) & (gy - Y0 < d + eta(gx))
    fx, fy = gx[fl], gy[fl]
    e = eta(fx)
    u = c0 * e
    # vertical velocity making the depth-uniform u divergence-free: w = -z du/dx
    dedx = -2.0 * k * e * np.tanh(k * (fx - X0 - x0)) if A > 0 else np.zeros_like(e)
    w = -(fy - Y0) * c0 * dedx
    thick_v = thick * math.sqrt(1.0 + slope * slope)
    inbed = (fx - X0 > toe) & (fy - Y0 < yslope(fx) + thick_v)
    con = np.where(inbed & saline_beach, 0.5, -0.5)
    oden = np.where(con > 0, rho * p.rel_den, rho)
    # --- grains of the porous layer (same lattice)
    gsel = (gx - X0 > toe) & (gy - Y0 >= yslope(gx)) & (gy - Y0 < yslope(gx) + thick_v)
    bulk = 1800.0
    grains = {"x": gx[gsel].copy(), "y": gy[gsel].copy(),
              "mass": np.full(int(gsel.sum()), bulk * dx * dx), "rho": np.full(int(gsel.sum()), bulk)}
    # Pore-fluid particles sit on the same lattice as free fluid, so each one
    # carries the fluid mass of its lattice cell, phi*rho0*dx^2 (ovol = phi*dx^2):
    # then m/rho = dx^2 with rho = phi*rho0 as effpor sets it (porous.f90:188-190).
    phi = porosity_field(fx, fy, grains, p.h, por)
    ovol = phi * dx * dx
    pf = oden * (-g) * np.maximum(0.0, d + e - (fy - Y0))
    parts.append(_mk(fx, fy, np.full(len(fx), abi.TID_FLUID), oden * ovol, phi * oden, oden,
                     ovol, con, vx=u, vy=w, p=pf))
    st = _cat(parts)
    p.wc_c0 = 10.0 * math.sqrt(-g * d)
    p.wc_ysurf = Y0 + d
    _grid_for(p, X0 + max(L, Lw) + (layers + 1) * dx, Y0 + H + 0.3)
    if wcsph:
        p, st = to_wcsph(p, st)
    return p, st, grains


def to_wcsph(p, st):
    """WCSPH set-up of a beach scene: every fluid particle carries the full
    lattice mass rho0 dl^2 and the Tait density of its pressure; the
    corrected continuity (the form as written is unstable)."""
    p = abi.Params.from_buffer_copy(p)
    st = dict(st)
    p.wc_form = 1
    dx, rho = p.dl, p.rho
    fl = st["tid"] == abi.TID_FLUID
    st["ovol"] = np.where(fl, dx * dx, st["ovol"])
    st["mass"] = np.where(fl, st["oden"] * dx * dx, st["mass"])
    c2 = p.wc_c0 ** 2
    st["rho"] = np.where(fl, rho * (st["p"] * p.wc_gamma / (rho * c2) + 1.0) ** (1.0 / p.wc_gamma), st["rho"])
    return p, st


def lattice_scene(n=1000, dx=1e-3, jitter=0.25, seed=20261203, layers=3, hfac=1.3):
    """Jittered square lattice of n x n particles with wall + ghost layers on
    three sides and a free top row (standalone search + PPE workload)."""
    rng = np.random.default_rng(seed)
    p = abi.default_params()
    p.h = hfac * dx
    p.dl = dx
    p.scalar_on = 0
    X0 = Y0 = (layers + 0.5) * dx
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    fx = X0 + (ii.ravel() + 0.5) * dx + rng.uniform(-jitter, jitter, n * n) * dx
    fy = Y0 + (jj.ravel() + 0.5) * dx + rng.uniform(-jitter, jitter, n * n) * dx
    wx, wy, wt = [], [], []
    for lay in range(layers):
        tid = abi.TID_WALL if lay == 0 else abi.TID_GHOST
        xb = X0 + (np.arange(-layers, n + layers) + 0.5) * dx
        wx.append(xb); wy.append(np.full_like(xb, Y0 - (lay + 0.5) * dx))
        wt.append(np.where((xb > X0) & (xb < X0 + n * dx), tid, abi.TID_GHOST))
        yl = Y0 + (np.arange(n + 2) + 0.5) * dx
        wx.append(np.full_like(yl, X0 - (lay + 0.5) * dx)); wy.append(yl); wt.append(np.full(len(yl), tid))
        wx.append(np.full_like(yl, X0 + n * dx + (lay + 0.5) * dx)); wy.append(yl); wt.append(np.full(len(yl), tid))
    wx = np.concatenate(wx); wy = np.concatenate(wy); wt = np.concatenate(wt)
    fmass = p.rho * dx * dx
    parts = [_mk(wx, wy, wt, fmass, p.rho, 0.0, 0.0, 0.0),
             _mk(fx, fy, np.full(n * n, abi.TID_FLUID), fmass, p.rho, p.rho, dx * dx, -0.5)]
    st = _cat(parts)
    p.wc_c0 = 10.0 * math.sqrt(-p.g * n * dx)
    p.wc_ysurf = Y0 + n * dx
    _grid_for(p, X0 + (n + layers + 1) * dx, Y0 + (n + 4) * dx)
    grains = {"x": np.zeros(0), "y": np.zeros(0), "mass": np.zeros(0), "rho": np.zeros(0)}
    return p, st, grains


def batch_scenes(count=64, seed=20261203, precision=abi.PREC_MIXED, dx_range=(0.005, 0.02), wcsph=False,
                 dx=None):
    """Seeded beach scenes: slope 1:5..1:20, amplitude 0.02..0.10 m,
    porosity 0.3..0.5, dx log-uniform in dx_range (uneven sizes) or the
    given list of dx."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        slope = 1.0 / rng.uniform(5.0, 20.0)
        A = rng.uniform(0.02, 0.10)
        por = rng.uniform(0.3, 0.5)
        d = float(np.exp(rng.uniform(np.log(dx_range[0]), np.log(dx_range[1]))))
        if dx is not None:
            d = float(dx[k])
        out.append(beach_scene(dx=d, slope=slope, A=A, por=por, precision=precision, wcsph=wcsph))
    return out


# particles of a beach scene per unit 1/dx^2 (fluid + walls, A = 0.06, 1:10)
BEACH_N_DX2 = 712460 * 0.00125 ** 2


def dx_for_particles(n):
    """Lattice spacing that gives a beach scene of about n particles."""
    return float(np.sqrt(BEACH_N_DX2 / n))


def cell_of(p, x, y):
    """(i, j) of the interior cell that holds (x, y) by the half-open bounds
    of setup.f90:120-123 (xleft = (j-2) 4h, ytop = (celly - i) 4h), or None."""
    cw = 4.0 * p.h
    j = int(math.floor(x / cw)) + 2
    i = p.celly - 1 - int(math.floor(y / cw))
    for di in (0, -1, 1):
        for dj in (0, -1, 1):
            ii, jj = i + di, j + dj
            if ((jj - 2) * cw <= x < (jj - 1) * cw) and ((-ii + p.celly - 1) * cw <= y < (-ii + p.celly) * cw):
                if 2 <= ii <= p.celly - 1 and 2 <= jj <= p.cellx - 1:
                    return ii, jj
    return None


def with_inflow(p, st, ncol=5, ntemplate=2, entry_vel=-0.05, period=0.0, phase=0.0, release_gap=None):
    """An open-boundary buffer zone on the right of a scene's fluid, shaped as
    the reference's right-hand buffer (internal.f90:98-215): the last `ncol`
    fluid columns become buffer particles moving at entry_vel, the last
    `ntemplate` columns are the template (buffer1: column by column, top row
    first), the entry cells are the cells holding the zone, and buffer
    particles at or beyond 0.75 spacing left of the first template column are
    removed at an exchange (rv_buf_r).  Inserted particles take the lattice
    mass, rho, ovol and con = -0.5 (insert_buffer1).  With release_gap, buffer
    particles that move left of the zone's first column minus the gap become
    fluid (comp_pos, integrator.f90:865-872).  Changes st in place; returns
    the zone dict for set_inflow."""
    fl = st["tid"] == abi.TID_FLUID
    xr = np.round(st["x"] / p.dl * 8.0) / 8.0   # lattice columns (unjittered scenes)
    cols = np.unique(xr[fl])
    zone_cols, tmpl_cols = cols[-ncol:], cols[-ntemplate:]
    inz = fl & np.isin(xr, zone_cols)
    st["flags"] = st["flags"] | np.where(inz, abi.FLAG_BUFFER, 0).astype(np.uint8)
    st["vx"] = np.where(inz, entry_vel, st["vx"])
    st["vy"] = np.where(inz, 0.0, st["vy"])
    tq = np.nonzero(fl & np.isin(xr, tmpl_cols))[0]
    tq = tq[np.lexsort((-st["y"][tq], xr[tq]))]   # column by column, top row first
    cells = sorted({cell_of(p, st["x"][q], st["y"][q]) for q in np.nonzero(inz)[0]} - {None},
                   key=lambda c: (c[1], c[0]))
    dx = p.dl
    x_first = float(st["x"][inz].min())
    if release_gap is not None:
        p.buf_release_lo = float(st["x"][fl].min())
        p.buf_release_hi = x_first - release_gap
    return {"x": st["x"][tq].copy(), "y": st["y"][tq].copy(), "vx": np.full(len(tq), entry_vel),
            "vy": np.zeros(len(tq)), "p": st["p"][tq].copy(), "pid": None,
            "mass": p.rho * dx * dx, "rho": p.rho, "ovol": dx * dx, "con": -0.5,
            "period": period, "phase": phase, "remove_x": float(st["x"][tq].min()) - 0.75 * dx,
            "remove_side": 1, "cells": cells}
