"""Generate the golden fixtures of the reference itself: its own aquifer
scene (setup.f90 init, boundary.f90 gen_boundary, internal.f90 gen_fluid)
run through its own main program (main.f90:23-272) by the reference's
Fortran source, translated and compiled by oracle/ref_build.py (the MKL
solve replaced by the reference's own BiCGStab, solved to the recurrence
residual 1e-13; the recipe's docstring lists the patch).

    python tests/golden/make_ref_golden.py

Needs the reference tree (only in the build container).  Writes
ref_aquifer.npz with, for each dump, the particle state in the reference's
cell/slot order:
* schedule "all" -- 3 settling steps, the fluid at rest, 3 settling steps
  with the buffers, the salinity set-up, 4 production steps, with the two
  buffer zones exchanging every 4.5 ms and 8.5 ms (so the short run
  exchanges): dumps after the set-up (step 0) and at the end of each phase
  (steps 3, 6, 10);
* schedule "settle50" -- the first settling phase in full (50 steps):
  dump at step 50.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

REC = 22
NAMES = ["pid", "tid", "x", "y", "vx", "vy", "p", "rho", "mass", "con", "oden", "ovol", "buffer", "free",
         "porosity", "nut", "tke", "cell_j", "cell_i", "slot", "dt", "t"]
KEEP = {"tid": np.int8, "x": None, "y": None, "vx": None, "vy": None, "p": None, "rho": None, "mass": None,
        "con": None, "porosity": None, "nut": None, "buffer": np.int8, "free": np.int8, "cell_j": np.int32,
        "cell_i": np.int32}
SCHEDULES = {"all": ((3, 3, 4), (0.0045, 0.0085), (0, 3, 6, 10)), "settle50": ((50, 0, 0), None, (50,))}


def load_dump(path):
    with open(path, "rb") as f:
        b = f.read()
    n = int(np.frombuffer(b[:8], np.int64)[0])
    a = np.frombuffer(b[8:], np.float64).reshape(n, REC)
    return {k: a[:, i] for i, k in enumerate(NAMES)}


def main():
    import ref_build
    exe = ref_build.build()
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, (steps, periods, dumps) in SCHEDULES.items():
            pre = os.path.join(tmp, name)
            cmd = [exe, pre] + [str(s) for s in steps] + ["1000000"]
            if periods:
                cmd += [repr(periods[0]), repr(periods[1])]
            subprocess.check_call(cmd)
            for k in dumps:
                d = load_dump(f"{pre}_{k}.bin")
                for f, dt in KEEP.items():
                    out[f"{name}_{k}_{f}"] = d[f].astype(dt) if dt else d[f]
                out[f"{name}_{k}_t"] = np.array(d["t"][0])
                out[f"{name}_{k}_dt"] = np.array(d["dt"][0])
    np.savez_compressed(os.path.join(HERE, "ref_aquifer.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_aquifer.npz"))


if __name__ == "__main__":
    main()
