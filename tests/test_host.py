"""CPU tests of the host side: the C-ABI library loads and exports every
symbol include/beachslope.h declares, the ctypes mirror matches the C
struct layouts, and the synthetic scene generators have the named shapes.
No GPU compute is called here."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "beachslope.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(bs_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from beachslope_gb300 import build
    lib_path = build.build_library()
    lib = C.CDLL(lib_path)
    syms = declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_struct_layouts_match_c(tmp_path):
    from beachslope_gb300 import abi
    src = r'''
    #include <stdio.h>
    #include <stddef.h>
    #include "beachslope.h"
    int main(void) {
      printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(bs_params), sizeof(bs_state), sizeof(bs_grains),
             sizeof(bs_scene_info), offsetof(bs_params, ppe_tol), offsetof(bs_state, coff),
             offsetof(bs_scene_info, err_bits));
      return 0; }
    '''
    tmp = str(tmp_path)
    c_file = os.path.join(tmp, "layout_check.c")
    exe = os.path.join(tmp, "layout_check")
    with open(c_file, "w") as f:
        f.write(src)
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c_file, "-o", exe])
    vals = list(map(int, subprocess.check_output([exe]).split()))
    assert vals == [C.sizeof(abi.Params), C.sizeof(abi.State), C.sizeof(abi.Grains), C.sizeof(abi.SceneInfo),
                    abi.Params.ppe_tol.offset, abi.State.coff.offset, abi.SceneInfo.err_bits.offset]


def test_beach_scene_config1_shape():
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.01)
    fluid = int((st["tid"] == 3).sum())
    walls = int((st["tid"] != 3).sum())
    assert 10_000 < fluid < 13_500
    assert 1_500 < walls < 4_000
    assert p.h == pytest.approx(0.013) and p.dt == 1e-4 and p.ppe_tol == 1e-8
    assert p.por == pytest.approx(0.40) and p.d50 == pytest.approx(0.005)
    assert len(gr["x"]) > 0
    # three wall layers, the one touching the fluid fixed (tid 1)
    assert set(np.unique(st["tid"])) == {1, 2, 3}
    # every particle lies inside the interior cell grid (columns/rows 2..n-1)
    cw = 4 * p.h
    assert st["x"].min() > 0 and st["y"].min() > 0
    assert st["x"].max() < (p.cellx - 2) * cw and st["y"].max() < (p.celly - 2) * cw


def test_beach_scene_pore_mass_consistent():
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.02)
    f = st["tid"] == 3
    phi = st["rho"][f] / st["oden"][f]
    # m / rho = dx^2 for every fluid particle (pore fluid carries phi*rho0*dx^2)
    np.testing.assert_allclose(st["mass"][f] / st["rho"][f], p.dl ** 2, rtol=1e-12)
    assert phi.min() == pytest.approx(p.por, rel=1e-9) and phi.max() == 1.0


def test_lattice_scene_shape():
    from beachslope_gb300 import scene
    p, st, gr = scene.lattice_scene(n=50, dx=1e-3)
    f = st["tid"] == 3
    assert f.sum() == 2500
    dx = p.dl
    X0 = 3.5 * dx
    i = np.round((st["x"][f] - X0) / dx - 0.5)
    assert np.max(np.abs(st["x"][f] - (X0 + (i + 0.5) * dx))) <= 0.25 * dx + 1e-15


def test_batch_scenes_uneven():
    from beachslope_gb300 import scene
    out = scene.batch_scenes(count=4, seed=7, dx_range=(0.02, 0.04))
    sizes = [len(s[1]["x"]) for s in out]
    assert len(set(sizes)) > 1
    slopes = [s[0].dl for s in out]
    assert all(0.02 <= d <= 0.04 for d in slopes)


def test_download_into_buffers_host_logic():
    """abi.state_out with caller buffers: views of their first n rows, and
    a clear error for buffers that are too short or of the wrong type."""
    import numpy as np
    from beachslope_gb300 import abi
    n = 10
    into = {f: np.zeros(n + 5) for f in abi.STATE_FIELDS_F64}
    into.update({f: np.zeros(n + 5, np.int32) for f in abi.STATE_FIELDS_I32})
    into["flags"] = np.zeros(n + 5, np.uint8)
    st, out = abi.state_out(n, False, into)
    assert st.n == n and all(len(v) == n for v in out.values())
    assert all(np.shares_memory(out[f], into[f]) for f in out)
    short = dict(into, x=np.zeros(n - 1))
    with pytest.raises(ValueError):
        abi.state_out(n, False, short)
    wrong = dict(into, pid=np.zeros(n + 5))
    with pytest.raises(ValueError):
        abi.state_out(n, False, wrong)


def test_inflow_and_field_structs():
    """abi.inflow_in / fields_in: the C structs carry the dict's arrays and
    scalars; None clears a zone; absent fields stay null pointers."""
    import numpy as np
    from beachslope_gb300 import abi
    assert abi.inflow_in(None).n == 0 and abi.inflow_in(None).ncells == 0
    z = {"x": [1.0, 2.0], "y": [3.0, 4.0], "vx": [0.1, 0.1], "vy": [0.0, 0.0], "p": [5.0, 6.0],
         "pid": None, "mass": 0.08, "rho": 1000.0, "ovol": 8e-5, "con": -0.5, "period": 391.0,
         "phase": 8.05, "remove_x": 3.18, "remove_side": 1, "cells": [(5, 44), (6, 44)]}
    s = abi.inflow_in(z)
    assert s.n == 2 and s.ncells == 2 and s.remove_side == 1 and not s.pid
    assert [s.x[k] for k in range(2)] == [1.0, 2.0] and [s.p[k] for k in range(2)] == [5.0, 6.0]
    assert [(s.cell_i[k], s.cell_j[k]) for k in range(2)] == [(5, 44), (6, 44)]
    assert (s.mass, s.rho, s.con, s.period, s.phase, s.remove_x) == (0.08, 1000.0, -0.5, 391.0, 8.05, 3.18)
    f = abi.fields_in({"vx": np.arange(3.0), "con": np.ones(3)})
    assert f.n == 3 and f.vx[2] == 2.0 and f.con[0] == 1.0
    assert not f.vy and not f.p and not f.mass
