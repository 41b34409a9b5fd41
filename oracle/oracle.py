"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the C++ FP64 oracle.

The oracle (bs_oracle.cpp) restates the reference's ISPH step; this module
builds it (g++, OpenMP) into oracle/_build/ and exposes a small class used by
tests/, the smoke check and bench.py's CPU baseline.  The product never
imports it.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libbsoracle.so")
SRC = [os.path.join(HERE, "bs_oracle.cpp")]
DEPS = SRC + [os.path.join(HERE, "bs_oracle.h"),
              os.path.join(HERE, "..", "include", "beachslope.h")]

STAGES = dict(projection=1, cellshift=2, cellshiftalt=3, resetid=4, neighbour=5, effpor=6,
              eddyvis=7, int_vel=8, ppe_assemble=9, ppe_solve=10, comp_vel=11, comp_pos=12,
              freesurf=13, opt2_shift=14, densityupdate=15, timestep=16, scalar_substep=17,
              prime=18, calmasscons=19, updateden=20, dentopress=21, presstoden=22,
              wall_pressure=23, effpor_keep=24, boun_vel=25, ghost=26, ghost_mls=27, prime_setup=28)


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB):
        t = os.path.getmtime(LIB)
        if all(os.path.getmtime(d) <= t for d in DEPS):
            return LIB
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           "-o", LIB + ".tmp"] + SRC
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp = C.c_void_p
        L.or_create.restype = vp
        L.or_create.argtypes = [vp, vp, vp]
        L.or_destroy.argtypes = [vp]
        L.or_n.argtypes = [vp]
        L.or_get.argtypes = [vp, vp]
        L.or_info.argtypes = [vp, vp]
        L.or_neighbours.argtypes = [vp, C.c_int32, vp, vp, vp, vp, vp]
        L.or_matrix.argtypes = [vp, C.c_int32, vp, vp, vp]
        L.or_stage.argtypes = [vp, C.c_int32]
        L.or_ppe_solve.argtypes = [vp, C.c_double, C.c_int32, C.c_int32, vp, vp]
        L.or_step.argtypes = [vp, C.c_int32]
        L.or_wcsph_step.argtypes = [vp, C.c_int32]
        L.or_write_combined.argtypes = [vp, C.c_char_p, C.c_char_p]
        L.or_set_pressure.argtypes = [vp, vp]
        L.or_set_inflow.argtypes = [vp, C.c_int32, vp]
        L.or_step_flags.argtypes = [vp, C.c_int32, C.c_int32]
        L.or_set_fields.argtypes = [vp, vp]
        L.or_set_time.argtypes = [vp, C.c_double]
        L.or_collision_shift.argtypes = [vp, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_double]
        L.or_buffer_exchange.argtypes = [vp, C.c_int32]
        L.or_set_threads.argtypes = [C.c_int]
        L.or_ppe_fgmres.argtypes = [vp, C.c_double, C.c_int32, C.c_int32, C.c_int32, vp, vp]
        L.or_fgmres_csr.argtypes = [C.c_int32, vp, vp, vp, vp, vp, C.c_double, C.c_int32, C.c_int32,
                                    C.c_int32, vp, vp]
        L.or_bicgstab_csr.argtypes = [C.c_int32, vp, vp, vp, vp, vp, C.c_double, C.c_int32,
                                      C.c_int32, vp, vp]
        L.or_Wab.restype = C.c_double
        L.or_Wab.argtypes = [C.c_double, C.c_double]
        L.or_Wo.restype = C.c_double
        L.or_Wo.argtypes = [C.c_double]
        L.or_gradW.argtypes = [C.c_double] * 6 + [vp, vp]
        L.or_invert2.argtypes = [vp]
        L.or_vis.restype = C.c_double
        L.or_vis.argtypes = [C.c_double]
        _lib = L
    return _lib


def _abi():
    mod = sys.modules.get("beachslope_gb300.abi")
    if mod is None:
        sys.path.insert(0, os.path.join(HERE, ".."))
        import __graft_entry__ as ge  # noqa: E402
        mod = ge.load_package().abi
    return mod


class Oracle:
    """One scene on the CPU oracle."""

    def __init__(self, params, state, grains=None):
        abi = _abi()
        self.abi = abi
        self.params = params
        self._st = abi.state_in(state)
        self._gr = abi.grains_in(grains) if grains is not None and len(grains["x"]) else None
        self.h = lib().or_create(C.byref(params), C.byref(self._st),
                                 C.byref(self._gr) if self._gr is not None else None)
        if not self.h:
            raise RuntimeError("or_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_destroy(self.h)
            self.h = None

    @property
    def n(self):
        return lib().or_n(self.h)

    def get(self):
        st, out = self.abi.state_out(self.n)
        lib().or_get(self.h, C.byref(st))
        return out

    def info(self):
        si = self.abi.SceneInfo()
        lib().or_info(self.h, C.byref(si))
        return si.as_dict()

    def neighbours(self, kmax=64):
        n = self.n
        counts = np.zeros(n, np.int32)
        idx = np.full((n, kmax), -1, np.int32)
        dist = np.zeros((n, kmax))
        kx = np.zeros((n, kmax))
        ky = np.zeros((n, kmax))
        rc = lib().or_neighbours(self.h, kmax, counts.ctypes.data, idx.ctypes.data, dist.ctypes.data,
                                 kx.ctypes.data, ky.ctypes.data)
        if rc != 0:
            raise RuntimeError("neighbour list longer than kmax")
        return counts, idx, dist, kx, ky

    def matrix(self, kmax=64):
        n = self.n
        diag = np.zeros(n)
        off = np.zeros((n, kmax))
        rhs = np.zeros(n)
        rc = lib().or_matrix(self.h, kmax, diag.ctypes.data, off.ctypes.data, rhs.ctypes.data)
        if rc != 0:
            raise RuntimeError("matrix not assembled")
        return diag, off, rhs

    def stage(self, name):
        rc = lib().or_stage(self.h, STAGES[name])
        return rc

    def ppe_solve(self, tol, maxit=20000, rule=0):
        it = C.c_int32(0)
        rr = C.c_double(0)
        rc = lib().or_ppe_solve(self.h, tol, maxit, rule, C.byref(it), C.byref(rr))
        return rc, it.value, rr.value

    def ppe_fgmres(self, tol, maxit=150, restart=150, rule=2):
        it = C.c_int32(0)
        rr = C.c_double(0)
        rc = lib().or_ppe_fgmres(self.h, tol, maxit, restart, rule, C.byref(it), C.byref(rr))
        return rc, it.value, rr.value

    def step(self, n=1):
        lib().or_step(self.h, n)

    def wcsph_step(self, n=1):
        lib().or_wcsph_step(self.h, n)

    def write_combined(self, fluid_path, buffer_path=None):
        return lib().or_write_combined(self.h, fluid_path.encode(),
                                       buffer_path.encode() if buffer_path else None)

    def set_inflow(self, zone_index, zone):
        z = self.abi.inflow_in(zone)
        rc = lib().or_set_inflow(self.h, zone_index, C.byref(z))
        if rc != 0:
            raise RuntimeError(f"or_set_inflow failed ({rc})")

    def step_flags(self, n, flags):
        return lib().or_step_flags(self.h, int(n), int(flags))

    def set_fields(self, fields):
        st = self.abi.fields_in(fields)
        rc = lib().or_set_fields(self.h, C.byref(st))
        if rc != 0:
            raise RuntimeError(f"or_set_fields failed ({rc})")

    def set_time(self, t):
        lib().or_set_time(self.h, float(t))

    def buffer_exchange(self, zone_index):
        return lib().or_buffer_exchange(self.h, zone_index)

    def collision_shift(self, mode, prx, pry, brx, bry):
        """coll_pos_shift (mode 0) / coll_shift (mode 1)."""
        rc = lib().or_collision_shift(self.h, int(mode), prx, pry, brx, bry)
        if rc != 0:
            raise RuntimeError(f"or_collision_shift failed ({rc})")

    def set_pressure(self, p):
        p = np.ascontiguousarray(p, dtype=np.float64)
        lib().or_set_pressure(self.h, p.ctypes.data)


def set_threads(n):
    lib().or_set_threads(int(n))


def bicgstab_csr(row_ptr, col, val, b, x0, tol=1e-12, maxit=1000, rule=0):
    row_ptr = np.ascontiguousarray(row_ptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.array(x0, dtype=np.float64)
    it = C.c_int32(0)
    rr = C.c_double(0)
    rc = lib().or_bicgstab_csr(len(b), row_ptr.ctypes.data, col.ctypes.data, val.ctypes.data,
                               b.ctypes.data, x.ctypes.data, tol, maxit, rule, C.byref(it), C.byref(rr))
    return rc, x, it.value, rr.value


def fgmres_csr(row_ptr, col, val, b, x0, tol=1e-3, maxit=150, restart=150, rule=2):
    row_ptr = np.ascontiguousarray(row_ptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.array(x0, dtype=np.float64)
    it = C.c_int32(0)
    rr = C.c_double(0)
    rc = lib().or_fgmres_csr(len(b), row_ptr.ctypes.data, col.ctypes.data, val.ctypes.data, b.ctypes.data,
                             x.ctypes.data, tol, maxit, restart, rule, C.byref(it), C.byref(rr))
    return rc, x, it.value, rr.value


def Wab(r, h):
    return lib().or_Wab(r, h)


def Wo(h):
    return lib().or_Wo(h)


def gradW(xj, yj, xi, yi, r, h):
    wx = C.c_double()
    wy = C.c_double()
    lib().or_gradW(xj, yj, xi, yi, r, h, C.byref(wx), C.byref(wy))
    return wx.value, wy.value


def invert2(a):
    a = np.array(a, dtype=np.float64)
    lib().or_invert2(a.ctypes.data)
    return a


def vis(oden):
    return lib().or_vis(oden)
