"""Small hand-built scenes shared by the CPU and GPU tests."""
import numpy as np


def ghost_row_scene():
    """A fluid block left of a three-layer wall whose layers sit one cell
    column to the right of the fluid: the second-layer ghost's first (lowest
    row) neighbour is a fluid particle, the case where the reference keeps the
    row initialiser's val(1)=1.0 (isph.f90:125-128)."""
    from beachslope_gb300 import abi, scene
    p = abi.default_params()
    dx = 0.01
    p.h = 1.3 * dx
    p.dl = dx
    cw = 4 * p.h
    # fluid columns x = 0.060..0.100 (cell column 3), wall layers at 0.110,
    # 0.120, 0.130 (cell column 4): the ghost at 0.120 sees fluid at 0.100
    xs, ys = np.meshgrid(0.060 + np.arange(5) * dx, np.arange(8) * dx + cw + 0.005, indexing="ij")
    fx, fy = xs.ravel(), ys.ravel()
    wx0 = 0.110
    wx = np.repeat([wx0, wx0 + dx, wx0 + 2 * dx], 8)
    wy = np.tile(np.arange(8) * dx + cw + 0.005, 3)
    wt = np.repeat([1, 2, 2], 8)
    parts = [scene._mk(wx, wy, wt, p.rho * dx * dx, p.rho, 0.0, 0.0, 0.0),
             scene._mk(fx, fy, np.full(len(fx), 3), p.rho * dx * dx, p.rho, p.rho, dx * dx, -0.5)]
    st = scene._cat(parts)
    scene._grid_for(p, 4 * cw, 4 * cw)
    return p, st
