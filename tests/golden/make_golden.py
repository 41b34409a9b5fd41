"""Generate the golden fixtures of the oracle (C++ FP64 restatement of the
reference ISPH step) on small seeded scenes.

    python tests/golden/make_golden.py

Writes beach_dx004.npz (beach scene, dx = 0.04 m: state after the warm-up
and after 1 and 3 production steps, neighbour lists, PPE rows) and
lattice_n24.npz (24 x 24 jittered lattice: neighbour lists, PPE rows, and
the BiCGStab solution for a seeded N(0,1) source).  The inputs are stored
with the outputs so each fixture is self-contained.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

ge.load_package()
from beachslope_gb300 import abi, scene  # noqa: E402
from oracle import oracle  # noqa: E402

STATE_KEYS = ["x", "y", "vx", "vy", "p", "mass", "rho", "oden", "ovol", "con", "tid", "pid", "flags"]
OUT_KEYS = STATE_KEYS + ["porosity", "nut", "tke", "gradvx", "coff", "cell"]


def pack_nbr(o, K):
    c, idx, dist, kx, ky = o.neighbours(K)
    m = np.arange(K)[None, :] < c[:, None]
    return c, idx[m], dist[m], kx[m], ky[m]


def params_arrays(p):
    return {"param_" + k: np.array(v) for k, v in p.as_dict().items()}


def beach():
    p, st, gr = scene.beach_scene(dx=0.04)
    p.ppe_tol = 1e-13
    out = {("in_" + k): st[k] for k in STATE_KEYS}
    out.update({("grain_" + k): gr[k] for k in gr})
    out.update(params_arrays(p))
    o = oracle.Oracle(p, st, gr)
    o.stage("prime")
    s = o.get()
    out.update({("prime_" + k): s[k] for k in OUT_KEYS})
    c, idx, dist, kx, ky = pack_nbr(o, p.kmax)
    out.update(prime_nbr_count=c, prime_nbr_idx=idx, prime_nbr_dist=dist, prime_nbr_kx=kx, prime_nbr_ky=ky)
    o.step(1)
    s = o.get()
    out.update({("step1_" + k): s[k] for k in OUT_KEYS})
    out.update(step1_info=np.array([o.info()["ppe_iters"]]))
    o.step(2)
    s = o.get()
    out.update({("step3_" + k): s[k] for k in OUT_KEYS})
    np.savez_compressed(os.path.join(HERE, "beach_dx004.npz"), **out)
    print("beach", len(st["x"]), "particles")


def lattice():
    p, st, gr = scene.lattice_scene(n=24, dx=1e-3)
    p.ppe_tol = 1e-13
    out = {("in_" + k): st[k] for k in STATE_KEYS}
    out.update(params_arrays(p))
    o = oracle.Oracle(p, st, None)
    o.stage("neighbour")
    o.stage("effpor")
    o.stage("int_vel")
    o.stage("ppe_assemble")
    c, idx, dist, kx, ky = pack_nbr(o, p.kmax)
    d, off, rhs = o.matrix(p.kmax)
    m = np.arange(p.kmax)[None, :] < c[:, None]
    out.update(nbr_count=c, nbr_idx=idx, nbr_dist=dist, diag=d, off=off[m], rhs=rhs)
    s = o.get()
    out.update(order_pid=s["pid"], coff=s["coff"], gradvx=s["gradvx"])
    np.savez_compressed(os.path.join(HERE, "lattice_n24.npz"), **out)
    print("lattice", len(st["x"]), "particles")


if __name__ == "__main__":
    beach()
    lattice()
