"""combined, output.f90:188-222: the text output of the fluid particles
(F10.3 x, y, p; ES10.3 vx, vy; F10.5 con+0.5), in the reference's particle
order, from the oracle and from the library."""
import numpy as np
import pytest


def _parse(path):
    rows = []
    with open(path) as f:
        for line in f:
            assert len(line.rstrip("\n")) == 65, line   # 6 fields of 10 + 5 separators
            rows.append([line[k * 11:k * 11 + 10] for k in range(6)])
    return rows


def _num(col):
    return np.array([np.nan if "*" in v else float(v) for v in col])


def test_combined_format_and_values(oracle, tmp_path):
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.04)
    o = oracle.Oracle(p, st, gr)
    o.stage("prime")
    g = o.get()
    fl = (g["tid"] == 3) & ((g["flags"] & 4) == 0)
    path = str(tmp_path / "fluid.txt")
    o.write_combined(path, str(tmp_path / "buffer.txt"))
    rows = _parse(path)
    assert len(rows) == int(fl.sum())
    cols = list(zip(*rows))
    x, y, pr = _num(cols[0]), _num(cols[1]), _num(cols[2])
    vx, vy, c = _num(cols[3]), _num(cols[4]), _num(cols[5])
    # order: cell-major as the oracle's get() (columns of cells, rows, slots)
    assert np.all(np.abs(x - g["x"][fl]) <= 0.0005 + 1e-12)
    assert np.all(np.abs(y - g["y"][fl]) <= 0.0005 + 1e-12)
    assert np.all(np.abs(pr - g["p"][fl]) <= 0.0005 + 1e-9)
    assert np.all(np.abs(vx - g["vx"][fl]) <= 5e-4 * np.abs(g["vx"][fl]) + 1e-300)
    assert np.all(np.abs(c - (g["con"][fl] + 0.5)) <= 5e-6 + 1e-12)
    # ES10.3 looks as gfortran prints it; an F10.3 value that does not fit is asterisks
    assert all(v.strip()[1:2] == "." or v.strip()[2:3] == "." for v in cols[3])
    assert all(("E+" in v or "E-" in v) for v in cols[3])
    pp = g["p"].copy()
    pp[np.argmax(fl)] = 1.0e9
    o.set_pressure(pp)
    o.write_combined(path)
    assert _parse(path)[0][2] == "*" * 10


@pytest.mark.gpu
def test_combined_gpu_matches_oracle(api, oracle, tmp_path):
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.02)
    p.ppe_tol = 1e-13
    ctx = api.Context([p], [st], [gr])
    o = oracle.Oracle(p, st, gr)
    ctx.prime(); o.stage("prime")
    ctx.step(1); o.step(1)
    a, b = str(tmp_path / "gpu.txt"), str(tmp_path / "ref.txt")
    ctx.write_combined(a)
    o.write_combined(b)
    ra, rb = _parse(a), _parse(b)
    assert len(ra) == len(rb)
    A = np.array([_num(c) for c in zip(*ra)])
    B = np.array([_num(c) for c in zip(*rb)])
    # a field printed as asterisks (value does not fit F10.3) must be so in both
    assert np.array_equal(np.isnan(A), np.isnan(B))
    A, B = np.nan_to_num(A), np.nan_to_num(B)
    # same particles in the same order; values equal up to the last printed
    # digit (the pressure also within the step's 1e-8 relative parity)
    assert np.all(np.abs(A[:2] - B[:2]) <= 1.001e-3)
    assert np.all(np.abs(A[2] - B[2]) <= 1.001e-3 + 1e-7 * np.abs(B[2]))
    assert np.all(np.abs(A[3:5] - B[3:5]) <= 1.001e-3 * np.abs(B[3:5]) + 1e-12)
    assert np.all(np.abs(A[5] - B[5]) <= 1.001e-5)
    same = np.mean([ra[k] == rb[k] for k in range(len(ra))])
    assert same > 0.95   # almost every line identical as text
