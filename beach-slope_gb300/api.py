"""Host-side context over libbeachslope.so (the C-ABI in include/beachslope.h).

Mirrors the reference's per-step entry points (search, effpor, eddyvis,
int_vel, ppesolve, comp_vel, comp_pos, freesurf, opt2_shift, densityupdate,
timestep, scalart_anisotropic) as methods; every call goes through the
CUDA library.  Errors from the library raise BeachSlopeError.  There is no
CPU fallback: if the library cannot be loaded, importing this module fails.
"""
import ctypes as C
import os
import weakref

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libbeachslope.so")


class BeachSlopeError(RuntimeError):
    pass


def _load():
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libbeachslope.so not built ({LIB_PATH}); run __graft_entry__.build()")
    L = C.CDLL(LIB_PATH)
    vp = C.c_void_p
    i32 = C.c_int32
    sig = {
        "bs_params_default": (None, [vp]),
        "bs_set_device": (C.c_int, [i32]),
        "bs_create": (C.c_int, [i32, vp, vp, vp, C.POINTER(vp)]),
        "bs_destroy": (C.c_int, [vp]),
        "bs_upload": (C.c_int, [vp, i32, vp, vp]),
        "bs_set_scene": (C.c_int, [vp, i32, vp, vp, vp]),
        "bs_prime_scene": (C.c_int, [vp, i32]),
        "bs_write_combined": (C.c_int, [vp, i32, C.c_char_p, C.c_char_p]),
        "bs_download": (C.c_int, [vp, i32, vp]),
        "bs_download_async": (C.c_int, [vp, i32, vp]),
        "bs_download_wait": (C.c_int, [vp, i32, vp]),
        "bs_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(vp)]),
        "bs_host_free": (C.c_int, [vp]),
        "bs_scene_info_get": (C.c_int, [vp, i32, vp]),
        "bs_clear_errors": (C.c_int, [vp]),
        "bs_sync": (C.c_int, [vp]),
        "bs_last_error": (C.c_char_p, [vp]),
        "bs_get_neighbours": (C.c_int, [vp, i32, vp, vp, vp, vp, vp]),
        "bs_get_matrix": (C.c_int, [vp, i32, vp, vp, vp]),
        "bs_set_rhs": (C.c_int, [vp, i32, vp]),
        "bs_set_option": (C.c_int, [vp, C.c_char_p, C.c_double]),
        "bs_get_option": (C.c_int, [vp, C.c_char_p, C.POINTER(C.c_double)]),
        "bs_prime": (C.c_int, [vp]),
        "bs_prime_setup": (C.c_int, [vp]),
        "bs_scalar_substep": (C.c_int, [vp]),
        "bs_projection": (C.c_int, [vp]),
        "bs_cellshift": (C.c_int, [vp, i32]),
        "bs_search": (C.c_int, [vp]),
        "bs_porosity": (C.c_int, [vp]),
        "bs_eddy": (C.c_int, [vp]),
        "bs_int_vel": (C.c_int, [vp]),
        "bs_ppe_assemble": (C.c_int, [vp]),
        "bs_ppe_solve": (C.c_int, [vp]),
        "bs_comp_vel": (C.c_int, [vp]),
        "bs_comp_pos": (C.c_int, [vp]),
        "bs_free_surface": (C.c_int, [vp]),
        "bs_shift": (C.c_int, [vp]),
        "bs_density_update": (C.c_int, [vp]),
        "bs_timestep": (C.c_int, [vp]),
        "bs_step": (C.c_int, [vp, i32]),
        "bs_wcsph_continuity": (C.c_int, [vp]),
        "bs_wcsph_update_density": (C.c_int, [vp]),
        "bs_wcsph_eos": (C.c_int, [vp]),
        "bs_wcsph_pressure_to_density": (C.c_int, [vp]),
        "bs_wcsph_wall_pressure": (C.c_int, [vp]),
        "bs_wcsph_step": (C.c_int, [vp, i32]),
        "bs_bicgstab_csr": (C.c_int, [i32, vp, vp, vp, vp, vp, C.c_double, i32, i32, vp, vp]),
        "bs_bicgstab_csr_noalloc": (C.c_int, [i32, vp, vp, vp, vp, vp, C.c_double, i32, vp, vp, vp]),
        "bs_fgmres_csr": (C.c_int, [i32, vp, vp, vp, vp, vp, C.c_double, i32, i32, i32, vp, vp]),
        "bs_set_inflow": (C.c_int, [vp, i32, i32, vp]),
        "bs_ghost": (C.c_int, [vp, i32]),
        "bs_collision_shift": (C.c_int, [vp, i32, C.c_double, C.c_double, C.c_double, C.c_double]),
        "bs_step_flags": (C.c_int, [vp, i32, i32]),
        "bs_set_fields": (C.c_int, [vp, i32, vp]),
        "bs_set_time": (C.c_int, [vp, i32, C.c_double]),
        "bs_buffer_exchange": (C.c_int, [vp, i32, i32]),
        "bs_event_record": (C.c_int, [vp, i32]),
        "bs_event_elapsed_ms": (C.c_int, [vp, i32, i32, C.POINTER(C.c_float)]),
        "bs_kernel_timing": (C.c_int, [vp, C.c_uint64]),
        "bs_kernel_timing_get": (C.c_int, [vp, i32, C.POINTER(C.c_char_p), C.POINTER(i32),
                                           C.POINTER(C.c_double)]),
        "bs_launch_count": (C.c_int64, [vp]),
        "bs_measure_fp64_peak": (C.c_int, [C.POINTER(C.c_double)]),
        "bs_device_memory": (C.c_int, [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
        "bs_context_bytes": (C.c_int, [vp, C.POINTER(C.c_size_t)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


lib = _load()

STAGE_FUNCS = ["prime", "scalar_substep", "projection", "search", "porosity", "eddy", "int_vel",
               "ppe_assemble", "ppe_solve", "comp_vel", "comp_pos", "free_surface", "shift",
               "density_update", "timestep", "boun_vel"]


class Context:
    """A batch of scenes resident on the GPU."""

    def __init__(self, params, states, grains=None, capacity=None, tuning=None, grain_capacity=None):
        if not isinstance(params, (list, tuple)):
            params, states, grains = [params], [states], [grains]
        n = len(params)
        if grains is None:
            grains = [None] * n
        self.nscenes = n
        self.params = (abi.Params * n)(*params)
        caps = capacity or [len(s["x"]) for s in states]
        gcaps = grain_capacity or [len(g["x"]) if g is not None else 0 for g in grains]
        self._caps = (C.c_int32 * n)(*caps)
        self._gcaps = (C.c_int32 * n)(*gcaps)
        h = C.c_void_p()
        rc = lib.bs_create(n, self.params, self._caps, self._gcaps, C.byref(h))
        if rc != 0:
            raise BeachSlopeError(f"bs_create failed ({rc})")
        self.h = h
        for s in range(n):
            self.upload(s, states[s], grains[s])
        self.tuning = None
        if tuning == "auto":   # solver options picked by the autotuner for this size class
            from . import autotune
            self.tuning = autotune.apply(self, params[0].precision, sum(caps), n)
        elif isinstance(tuning, dict):
            for k, v in tuning.items():
                self.set_option(k, v)
            self.tuning = tuning

    def close(self):
        if getattr(self, "h", None):
            lib.bs_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, rc, what):
        if rc != 0:
            msg = lib.bs_last_error(self.h)
            raise BeachSlopeError(f"{what} failed ({rc}): {msg.decode() if msg else ''}")

    def upload(self, s, state, grains=None):
        st = abi.state_in(state)
        gr = abi.grains_in(grains) if grains is not None and len(grains["x"]) else None
        self._check(lib.bs_upload(self.h, s, C.byref(st), C.byref(gr) if gr is not None else None), "upload")

    def set_scene(self, s, params, state, grains=None):
        """Put another scene into slot s (its cell grid no larger than the
        slot's creation grid); the other slots keep running untouched."""
        st = abi.state_in(state)
        gr = abi.grains_in(grains) if grains is not None and len(grains["x"]) else None
        self.params[s] = abi.Params.from_buffer_copy(params)
        self._check(lib.bs_set_scene(self.h, s, C.byref(self.params[s]), C.byref(st),
                                     C.byref(gr) if gr is not None else None), "set_scene")

    def write_combined(self, fluid_path, buffer_path=None, s=0):
        """The reference's combined text output (output.f90:188-222) for scene s."""
        self._check(lib.bs_write_combined(self.h, s, fluid_path.encode(),
                                          buffer_path.encode() if buffer_path else None), "write_combined")

    def prime_setup(self):
        """Prime without the time-step rule (the reference's own set-up)."""
        self._check(lib.bs_prime_setup(self.h), "prime_setup")

    def prime_scene(self, s):
        """Prime slot s alone (the other slots are left exactly as they are)."""
        self._check(lib.bs_prime_scene(self.h, s), "prime_scene")

    def info(self, s=0):
        si = abi.SceneInfo()
        self._check(lib.bs_scene_info_get(self.h, s, C.byref(si)), "scene_info")
        return si.as_dict()

    def download(self, s=0, full=True, out=None):
        """Scene s's particle fields in the library's row order.  out: a dict
        from pinned_state() (or a previous download) to fill instead of new
        arrays; the result is views of its first n rows."""
        n = self.info(s)["n"]
        st, res = abi.state_out(n, full, out)
        self._check(lib.bs_download(self.h, s, C.byref(st)), "download")
        return res

    def capacity_rows(self, s=0):
        """Rows the library reserves for scene s (its capacity rounded up to 256)."""
        return (int(self._caps[s]) + 255) // 256 * 256

    def download_async(self, s=0, out=None):
        """Start a read-back of scene s that overlaps the steps submitted after
        it (bs_download_async); out: a pinned_state() dict of at least
        capacity_rows(s) rows.  Returns a handle for download_wait."""
        rows = self.capacity_rows(s)
        st, res = abi.state_out(rows, False, out)
        self._check(lib.bs_download_async(self.h, s, C.byref(st)), "download_async")
        return (s, st, res)

    def download_wait(self, handle):
        """Finish a read-back started by download_async: views of its n rows."""
        s, st, res = handle
        self._check(lib.bs_download_wait(self.h, s, C.byref(st)), "download_wait")
        return {k: v[:st.n] for k, v in res.items()}

    def neighbours(self, s=0):
        n = self.info(s)["n"]
        K = self.params[s].kmax
        counts = np.zeros(n, np.int32)
        idx = np.full((n, K), -1, np.int32)
        dist = np.zeros((n, K))
        kx = np.zeros((n, K))
        ky = np.zeros((n, K))
        self._check(lib.bs_get_neighbours(self.h, s, counts.ctypes.data, idx.ctypes.data, dist.ctypes.data,
                                          kx.ctypes.data, ky.ctypes.data), "get_neighbours")
        return counts, idx, dist, kx, ky

    def neighbour_counts(self, s=0):
        n = self.info(s)["n"]
        counts = np.zeros(n, np.int32)
        self._check(lib.bs_get_neighbours(self.h, s, counts.ctypes.data, None, None, None, None),
                    "get_neighbours")
        return counts

    def matrix(self, s=0):
        n = self.info(s)["n"]
        K = self.params[s].kmax
        diag = np.zeros(n)
        off = np.zeros((n, K))
        rhs = np.zeros(n)
        self._check(lib.bs_get_matrix(self.h, s, diag.ctypes.data, off.ctypes.data, rhs.ctypes.data),
                    "get_matrix")
        return diag, off, rhs

    def set_inflow(self, zone_index, zone, s=0):
        """Open-boundary buffer zone (0: buffer1, 1: buffer2) of scene s; see
        abi.inflow_in for the dict; None clears it."""
        z = abi.inflow_in(zone)
        self._check(lib.bs_set_inflow(self.h, s, zone_index, C.byref(z)), "set_inflow")

    def step_flags(self, n, flags):
        """The step without the parts the flags leave out (abi.STEP_*)."""
        self._check(lib.bs_step_flags(self.h, int(n), int(flags)), "step_flags")

    def set_fields(self, fields, s=0):
        """Overwrite vx, vy, p, mass, rho, oden, ovol, con (the keys given) in
        place, in download order."""
        st = abi.fields_in(fields)
        self._check(lib.bs_set_fields(self.h, s, C.byref(st)), "set_fields")

    def set_time(self, t, s=0):
        self._check(lib.bs_set_time(self.h, s, float(t)), "set_time")

    def ghost(self, use_mls=False):
        """comp_ghost + ghost_en (mls.f90:114-263); use_mls: the MLS branch."""
        self._check(lib.bs_ghost(self.h, 1 if use_mls else 0), "ghost")

    def collision_shift(self, mode, prx, pry, brx, bry):
        """coll_pos_shift (mode 0) / coll_shift (mode 1), part_shift.f90:193-410;
        prx .. bry: the half particle spacings prrealx, prrealy, brrealx, brrealy."""
        self._check(lib.bs_collision_shift(self.h, int(mode), float(prx), float(pry), float(brx), float(bry)),
                    "collision_shift")

    def buffer_exchange(self, zone_index, s=0):
        self._check(lib.bs_buffer_exchange(self.h, s, zone_index), "buffer_exchange")

    def set_option(self, name, value):
        self._check(lib.bs_set_option(self.h, name.encode(), float(value)), "set_option " + name)

    def get_option(self, name):
        v = C.c_double()
        self._check(lib.bs_get_option(self.h, name.encode(), C.byref(v)), "get_option " + name)
        return v.value

    def set_rhs(self, b, s=0):
        b = np.ascontiguousarray(b, np.float64)
        self._check(lib.bs_set_rhs(self.h, s, b.ctypes.data), "set_rhs")

    def stage(self, name):
        f = getattr(lib, "bs_" + name)
        self._check(f(self.h), name)

    def cellshift(self, alt=False):
        self._check(lib.bs_cellshift(self.h, 1 if alt else 0), "cellshift")

    def step(self, n=1):
        self._check(lib.bs_step(self.h, n), "step")

    def wcsph_step(self, n=1):
        """WCSPH step (continuity + Tait EOS instead of the PPE), n times."""
        self._check(lib.bs_wcsph_step(self.h, n), "wcsph_step")

    def sync(self):
        self._check(lib.bs_sync(self.h), "sync")

    def clear_errors(self):
        self._check(lib.bs_clear_errors(self.h), "clear_errors")

    def record(self, slot):
        self._check(lib.bs_event_record(self.h, slot), "event_record")

    def elapsed_ms(self, a, b):
        ms = C.c_float()
        self._check(lib.bs_event_elapsed_ms(self.h, a, b, C.byref(ms)), "event_elapsed")
        return ms.value

    def kernel_timing(self, mask=(1 << 64) - 1):
        self._check(lib.bs_kernel_timing(self.h, mask), "kernel_timing")

    def kernel_times(self):
        out = {}
        for k in range(64):
            name = C.c_char_p()
            cnt = C.c_int32()
            ms = C.c_double()
            if lib.bs_kernel_timing_get(self.h, k, C.byref(name), C.byref(cnt), C.byref(ms)) != 0:
                break
            if cnt.value:
                out[name.value.decode()] = (cnt.value, ms.value)
        return out

    def kernel_ids(self):
        """name -> id of every kernel the per-kernel timer knows."""
        out = {}
        for k in range(256):
            name = C.c_char_p()
            if lib.bs_kernel_timing_get(self.h, k, C.byref(name), None, None) != 0:
                break
            out[name.value.decode()] = k
        return out

    def launch_count(self):
        return int(lib.bs_launch_count(self.h))

    def device_bytes(self):
        """Device bytes the context holds."""
        v = C.c_size_t()
        self._check(lib.bs_context_bytes(self.h, C.byref(v)), "context_bytes")
        return int(v.value)


for _name in STAGE_FUNCS:
    def _mk(nm):
        def f(self):
            self.stage(nm)
        f.__name__ = nm
        return f
    setattr(Context, _name, _mk(_name))


def pinned_empty(n, dtype=np.float64):
    """A numpy array in page-locked host memory (bs_host_alloc), freed with
    the array: uploads from and downloads into it run at the host link's
    rate."""
    dt = np.dtype(dtype)
    nbytes = max(int(n) * dt.itemsize, 1)
    p = C.c_void_p()
    rc = lib.bs_host_alloc(nbytes, C.byref(p))
    if rc != 0 or not p.value:
        raise BeachSlopeError(f"bs_host_alloc({nbytes}) failed ({rc})")
    buf = (C.c_char * nbytes).from_address(p.value)
    weakref.finalize(buf, lib.bs_host_free, p.value)
    return np.frombuffer(buf, dtype=dt, count=int(n))


def pinned_state(n, full=False):
    """Pinned arrays for Context.download(out=...) of up to n rows."""
    out = {f: pinned_empty(n) for f in abi.STATE_FIELDS_F64 + (abi.EXTRA_F64 if full else [])}
    for f in abi.STATE_FIELDS_I32:
        out[f] = pinned_empty(n, np.int32)
    out["flags"] = pinned_empty(n, np.uint8)
    if full:
        out["coff"] = pinned_empty(4 * n).reshape(n, 4)
        out["cell"] = pinned_empty(n, np.int32)
    return out


def pinned_copy(state):
    """A copy of a state dict (upload input) in pinned memory."""
    out = {}
    for k, v in state.items():
        v = np.asarray(v)
        a = pinned_empty(v.size, v.dtype).reshape(v.shape)
        a[...] = v
        out[k] = a
    return out


def set_device(device):
    """Pick the CUDA device for contexts created afterwards (one rank per GPU)."""
    rc = lib.bs_set_device(int(device))
    if rc != 0:
        raise BeachSlopeError(f"bs_set_device({device}) failed ({rc})")


def device_memory():
    """(free, total) bytes of the current device."""
    f, t = C.c_size_t(), C.c_size_t()
    rc = lib.bs_device_memory(C.byref(f), C.byref(t))
    if rc != 0:
        raise BeachSlopeError(f"bs_device_memory failed ({rc})")
    return f.value, t.value


def measure_fp64_peak():
    """FP64 TFLOP/s of the current device (chains of dependent DFMAs on every SM)."""
    v = C.c_double()
    rc = lib.bs_measure_fp64_peak(C.byref(v))
    if rc != 0:
        raise BeachSlopeError(f"bs_measure_fp64_peak failed ({rc})")
    return v.value


def bicgstab_csr(row_ptr, col, val, b, x0, tol=1e-12, maxit=1000, rule=abi.STOP_RELRES):
    """solvertest.f90's path: BiCGStab on a host CSR system, solved on the GPU."""
    row_ptr = np.ascontiguousarray(row_ptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.array(x0, dtype=np.float64)
    it = C.c_int32()
    rr = C.c_double()
    rc = lib.bs_bicgstab_csr(len(b), row_ptr.ctypes.data, col.ctypes.data, val.ctypes.data, b.ctypes.data,
                             x.ctypes.data, tol, maxit, rule, C.byref(it), C.byref(rr))
    return rc, x, it.value, rr.value


def fgmres_csr(row_ptr, col, val, b, x0, tol=1e-3, maxit=150, restart=150, rule=abi.STOP_R0):
    """fgmres (solver.f90:306-350): restarted GMRES on a host CSR system,
    solved on the GPU; defaults are the reference's MKL settings."""
    row_ptr = np.ascontiguousarray(row_ptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.array(x0, dtype=np.float64)
    it = C.c_int32()
    rr = C.c_double()
    rc = lib.bs_fgmres_csr(len(b), row_ptr.ctypes.data, col.ctypes.data, val.ctypes.data, b.ctypes.data,
                           x.ctypes.data, tol, maxit, restart, rule, C.byref(it), C.byref(rr))
    return rc, x, it.value, rr.value


def bicgstab_csr_noalloc(n, d_row_ptr, d_col, d_val, d_b, d_x, tol=1e-12, maxit=1000, stream=None):
    """BiCGStab on a CSR system already in device memory (integer device
    addresses), allocating nothing; see bs_bicgstab_csr_noalloc in
    include/beachslope.h for the limits.  Returns (status, iterations, relres)."""
    it = C.c_int32()
    rr = C.c_double()
    rc = lib.bs_bicgstab_csr_noalloc(int(n), d_row_ptr, d_col, d_val, d_b, d_x, float(tol), int(maxit), stream,
                                     C.byref(it), C.byref(rr))
    return rc, it.value, rr.value
