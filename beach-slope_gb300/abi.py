"""ctypes mirror of include/beachslope.h (structs and constants).

The C-ABI replaces the reference's module globals (initialize.f90:54-69) with
a context plus caller-owned SoA host buffers; these classes are the Python
view of those buffers, backed by numpy arrays.
"""
import ctypes as C

import numpy as np

BS_OK = 0
BS_E_ARG, BS_E_CUDA, BS_E_NOMEM, BS_E_CAPACITY = -1, -2, -3, -4
BS_E_NOTCONV, BS_E_NONFINITE, BS_E_DOMAIN, BS_E_STATE = -5, -6, -7, -8

ERR_BITS = {
    0x01: "neighbour overflow",
    0x02: "zero PPE diagonal",
    0x04: "solver breakdown",
    0x08: "not converged",
    0x10: "non-finite",
    0x20: "lost particle",
    0x40: "zero shift",
    0x80: "no neighbour",
}

TID_WALL, TID_GHOST, TID_FLUID = 1, 2, 3
FLAG_FREE, FLAG_VICINITY, FLAG_BUFFER = 0x01, 0x02, 0x04
PREC_FP64, PREC_MIXED = 0, 1
STOP_RELRES, STOP_REFERENCE, STOP_R0 = 0, 1, 2
SOLVER_BICGSTAB, SOLVER_FGMRES = 0, 1
STEP_SCALAR, STEP_BUFFERS, STEP_DENSITY, STEP_EDDY_END, STEP_ALL = 0x1, 0x2, 0x4, 0x8, 0xF

_d = C.c_double
_i = C.c_int32
_pd = C.POINTER(C.c_double)
_pi = C.POINTER(C.c_int32)
_pu8 = C.POINTER(C.c_uint8)


class Params(C.Structure):
    _fields_ = [
        ("h", _d), ("dl", _d), ("cellx", _i), ("celly", _i),
        ("dt", _d), ("t0", _d), ("adaptive_dt", _i), ("scalar_on", _i),
        ("rho", _d), ("rhomin", _d), ("rhomax", _d), ("rel_den", _d), ("g", _d),
        ("mu", _d), ("tschmidt", _d),
        ("por", _d), ("lamk", _d), ("d50", _d),
        ("lamfs", _d), ("maxdivr", _d), ("csh", _d), ("maxshift", _d), ("sig1", _d),
        ("xlcutoff", _d), ("ytcutoff", _d),
        ("ppe_tol", _d), ("ppe_maxit", _i), ("ppe_stop", _i), ("precision", _i),
        ("kmax", _i), ("mixed_inner_tol", _d), ("mixed_max_outer", _i), ("ppe_precond", _i),
        ("wc_c0", _d), ("wc_gamma", _d), ("wc_delta", _d), ("wc_ysurf", _d), ("wc_form", _i), ("wc_pad", _i),
        ("ppe_solver", _i), ("ppe_restart", _i),
        ("buf_release_lo", _d), ("buf_release_hi", _d),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def default_params():
    """Reference defaults (initialize.f90:21-81, porous.f90:111)."""
    p = Params()
    p.h = 0.013
    p.dl = 0.01
    p.cellx = p.celly = 0
    p.dt = 1e-4
    p.t0 = 0.0
    p.adaptive_dt = 0
    p.scalar_on = 1
    p.rho = 1000.0
    p.rhomin = 1000.0
    p.rel_den = 1.025
    p.rhomax = p.rho * p.rel_den
    p.g = -9.81
    p.mu = 0.001
    p.tschmidt = 1.0
    p.por = 0.38
    p.lamk = 600.0
    p.d50 = 0.00102
    p.lamfs = 0.80
    p.maxdivr = 2.0
    p.csh = 0.50
    p.maxshift = 0.1
    p.sig1 = 0.20
    p.xlcutoff = -1e300
    p.ytcutoff = 1e300
    p.ppe_tol = 1e-8
    p.ppe_maxit = 5000
    p.ppe_stop = STOP_RELRES
    p.precision = PREC_FP64
    p.kmax = 48
    p.mixed_inner_tol = 1e-3
    p.mixed_max_outer = 0   # 0: the mixed mode solves the PPE with the FP64 BiCGStab
    p.ppe_precond = 1       # multigrid V-cycle preconditioner
    p.wc_c0 = 0.0           # set per scene (10 sqrt(g depth))
    p.wc_gamma = 7.0        # t_gam, initialize.f90:46
    p.wc_delta = 0.1        # delt, initialize.f90:40
    p.wc_ysurf = 0.0        # set per scene (still-water level)
    p.ppe_solver = 0        # BiCGStab
    p.ppe_restart = 150     # FGMRES restart length (MKL's default in the reference's call)
    p.buf_release_lo = 1e300    # comp_pos buffer release window (empty: never)
    p.buf_release_hi = -1e300
    return p


STATE_FIELDS_F64 = ["x", "y", "vx", "vy", "p", "mass", "rho", "oden", "ovol", "con"]
STATE_FIELDS_I32 = ["tid", "pid"]
EXTRA_F64 = ["xs", "ys", "vxs", "vys", "porosity", "resx", "resy", "nut", "tke",
             "varts", "gradvx", "vel", "cdiff"]


class State(C.Structure):
    _fields_ = [("n", _i)] + [(f, _pd) for f in STATE_FIELDS_F64] + \
        [("tid", _pi), ("pid", _pi), ("flags", _pu8)] + \
        [(f, _pd) for f in EXTRA_F64] + [("coff", _pd), ("cell", _pi)]


class Grains(C.Structure):
    _fields_ = [("n", _i), ("x", _pd), ("y", _pd), ("mass", _pd), ("rho", _pd)]


class Inflow(C.Structure):
    _fields_ = [("n", _i), ("x", _pd), ("y", _pd), ("vx", _pd), ("vy", _pd), ("p", _pd), ("pid", _pi),
                ("mass", _d), ("rho", _d), ("ovol", _d), ("con", _d), ("period", _d), ("phase", _d),
                ("remove_x", _d), ("remove_side", _i), ("ncells", _i), ("cell_i", _pi), ("cell_j", _pi)]


def inflow_in(zone):
    """bs_inflow from a dict: template arrays x, y, vx, vy, p (pid optional),
    scalars mass, rho, ovol, con, period, phase, remove_x, remove_side and
    cells = [(i, j), ...] (1-based, dpcell(i, j)).  None clears the zone."""
    z = Inflow()
    if zone is None:
        return z
    keep = {k: np.ascontiguousarray(zone[k], dtype=np.float64) for k in ("x", "y", "vx", "vy", "p")}
    z.n = int(len(keep["x"]))
    for k in ("x", "y", "vx", "vy", "p"):
        setattr(z, k, _ptr(keep[k], C.c_double))
    if zone.get("pid") is not None:
        keep["pid"] = np.ascontiguousarray(zone["pid"], dtype=np.int32)
        z.pid = _ptr(keep["pid"], C.c_int32)
    for k in ("mass", "rho", "ovol", "con", "period", "phase", "remove_x"):
        setattr(z, k, float(zone[k]))
    z.remove_side = int(zone["remove_side"])
    cells = np.asarray(zone["cells"], dtype=np.int32).reshape(-1, 2)
    keep["ci"] = np.ascontiguousarray(cells[:, 0])
    keep["cj"] = np.ascontiguousarray(cells[:, 1])
    z.ncells = int(len(cells))
    z.cell_i = _ptr(keep["ci"], C.c_int32)
    z.cell_j = _ptr(keep["cj"], C.c_int32)
    z._keep = keep
    return z


class SceneInfo(C.Structure):
    _fields_ = [("n", _i), ("solsteps", _i), ("ppe_iters", _i), ("ppe_outer", _i),
                ("dt", _d), ("dtsol", _d), ("t", _d), ("umax", _d), ("numax", _d),
                ("ppe_relres", _d), ("err_bits", C.c_uint32), ("pad0", _i)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad0"}


def _ptr(a, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


def state_in(arrs):
    """bs_state pointing at a dict of numpy arrays (upload view).  Keeps refs."""
    n = int(len(arrs["x"]))
    keep = {}
    st = State()
    st.n = n
    for f in STATE_FIELDS_F64:
        keep[f] = np.ascontiguousarray(arrs[f], dtype=np.float64)
        setattr(st, f, _ptr(keep[f], C.c_double))
    for f in STATE_FIELDS_I32:
        keep[f] = np.ascontiguousarray(arrs[f], dtype=np.int32)
        setattr(st, f, _ptr(keep[f], C.c_int32))
    keep["flags"] = np.ascontiguousarray(arrs.get("flags", np.zeros(n, np.uint8)), dtype=np.uint8)
    st.flags = _ptr(keep["flags"], C.c_uint8)
    st._keep = keep
    return st


def fields_in(fields):
    """bs_state carrying the given in-place fields (bs_set_fields)."""
    keys = ("vx", "vy", "p", "mass", "rho", "oden", "ovol", "con")
    keep = {k: np.ascontiguousarray(fields[k], dtype=np.float64) for k in keys if k in fields}
    st = State()
    st.n = int(len(next(iter(keep.values()))))
    for k, v in keep.items():
        setattr(st, k, _ptr(v, C.c_double))
    st._keep = keep
    return st


def empty_state():
    """A scene with no particles (a free slot of a request loop)."""
    st = {f: np.zeros(0) for f in STATE_FIELDS_F64}
    st.update({f: np.zeros(0, np.int32) for f in STATE_FIELDS_I32})
    st["flags"] = np.zeros(0, np.uint8)
    return st


def state_out(n, full=True, into=None):
    """numpy arrays for a download and a bs_state pointing at them; into: a
    dict of arrays with at least n rows to fill instead (views returned)."""
    def arr(f, dtype, shape=()):
        if into is not None:
            a = into[f]
            if a.dtype != np.dtype(dtype) or len(a) < n or not a.flags.c_contiguous:
                raise ValueError(f"download buffer {f}: need {n} contiguous rows of {np.dtype(dtype)}")
            return a[:n]
        return np.zeros((n,) + shape, dtype)
    out = {}
    st = State()
    st.n = n
    for f in STATE_FIELDS_F64 + (EXTRA_F64 if full else []):
        out[f] = arr(f, np.float64)
        setattr(st, f, _ptr(out[f], C.c_double))
    for f in STATE_FIELDS_I32:
        out[f] = arr(f, np.int32)
        setattr(st, f, _ptr(out[f], C.c_int32))
    out["flags"] = arr("flags", np.uint8)
    st.flags = _ptr(out["flags"], C.c_uint8)
    if full:
        out["coff"] = arr("coff", np.float64, (4,))
        st.coff = _ptr(out["coff"], C.c_double)
        out["cell"] = arr("cell", np.int32)
        st.cell = _ptr(out["cell"], C.c_int32)
    st._keep = out
    return st, out


def grains_in(g):
    keep = {k: np.ascontiguousarray(g[k], dtype=np.float64) for k in ("x", "y", "mass", "rho")}
    gr = Grains()
    gr.n = int(len(keep["x"]))
    for k, v in keep.items():
        setattr(gr, k, _ptr(v, C.c_double))
    gr._keep = keep
    return gr
