"""CPU tests of the oracle (C++ FP64 restatement of the reference).

Pins: the reference's only known-answer test (solvertest.f90:10-19), the
analytic identities of the kernel/inverse/porosity routines, the cell
binning rule, and the committed golden fixtures (regression of the oracle).
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# solvertest.f90:10-19, converted to 0-based CSR; exact solution (1,2,3,4,5)
KAT_ROW = np.array([1, 4, 6, 8, 11, 14]) - 1
KAT_COL = np.array([1, 3, 4, 2, 4, 1, 3, 2, 3, 4, 1, 2, 5]) - 1
KAT_VAL = np.ones(13)
KAT_B = np.array([8.0, 6.0, 4.0, 9.0, 8.0])
KAT_X = np.array([1.0, 2.0, 3.0, 4.0, 5.0])


def test_solvertest_known_answer(oracle):
    rc, x, it, rr = oracle.bicgstab_csr(KAT_ROW, KAT_COL, KAT_VAL, KAT_B, np.ones(5), tol=1e-13)
    assert rc == 0
    np.testing.assert_allclose(x, KAT_X, rtol=0, atol=1e-10)
    assert rr < 1e-12


def test_solvertest_reference_stop_rule(oracle):
    # the reference's own stop (every |dx/(x+1e-5)| <= 1e-2, solver.f90:233-242)
    rc, x, it, rr = oracle.bicgstab_csr(KAT_ROW, KAT_COL, KAT_VAL, KAT_B, np.ones(5), tol=0.01, rule=1)
    assert rc == 0 and it >= 1
    np.testing.assert_allclose(x, KAT_X, rtol=5e-2)


def test_kernel_identities(oracle):
    h = 0.013
    # Wo is W at r=0 (kernel.f90:68-92)
    assert oracle.Wab(0.0, h) == pytest.approx(oracle.Wo(h), rel=1e-15)
    # compact support and continuity at r = h
    assert oracle.Wab(2 * h, h) == 0.0
    assert oracle.Wab(h * (1 - 1e-12), h) == pytest.approx(oracle.Wab(h, h), rel=1e-9)
    # gradient antisymmetry grad_i W_ij = -grad_j W_ji, and radial direction
    xi, yi, xj, yj = 0.10, 0.20, 0.11, 0.215
    r = np.hypot(xi - xj, yi - yj)
    gx, gy = oracle.gradW(xj, yj, xi, yi, r, h)
    hx, hy = oracle.gradW(xi, yi, xj, yj, r, h)
    assert gx == pytest.approx(-hx, rel=1e-15) and gy == pytest.approx(-hy, rel=1e-15)
    assert gx * (yi - yj) == pytest.approx(gy * (xi - xj), rel=1e-12)
    # gradient is the derivative of W (both branches)
    for rr in (0.4 * h, 1.5 * h):
        e = 1e-7 * h
        dW = (oracle.Wab(rr + e, h) - oracle.Wab(rr - e, h)) / (2 * e)
        gx, _ = oracle.gradW(0.0, 0.0, rr, 0.0, rr, h)
        assert gx == pytest.approx(dW, rel=1e-5)


def test_kernel_single_precision_literals(oracle):
    # 28.0*3.14 and 3.0*3.14 are evaluated in single precision (default REAL)
    h = 0.01
    c28 = float(np.float32(28.0) * np.float32(3.14))
    c3 = float(np.float32(3.0) * np.float32(3.14))
    wo = 0.1 * 4.0 * (10.0 / (c28 * h * h)) + 0.9 * 6.0 * (1.0 / (c3 * h * h))
    assert oracle.Wo(h) == pytest.approx(wo, rel=1e-15)


def test_invertmat2d(oracle):
    a = oracle.invert2([2.0, 1.0, 1.0, 3.0])
    inv = np.linalg.inv(np.array([[2.0, 1.0], [1.0, 3.0]]))
    np.testing.assert_allclose(a, [inv[0, 0], inv[0, 1], inv[1, 0], inv[1, 1]], rtol=1e-15)
    # singular or |det| < 1e-5 (single literal) -> identity (functions.f90:324-336)
    np.testing.assert_array_equal(oracle.invert2([1.0, 2.0, 2.0, 4.0]), [1, 0, 0, 1])
    np.testing.assert_array_equal(oracle.invert2([1e-3, 0.0, 0.0, 1e-3]), [1, 0, 0, 1])
    np.testing.assert_array_equal(oracle.invert2([np.nan, 0.0, 0.0, 1.0]), [1, 0, 0, 1])


def test_viscosity(oracle):
    assert oracle.vis(1000.0) == pytest.approx(1.002e-3, rel=1e-15)
    s = 25.0
    assert oracle.vis(1025.0) == pytest.approx((1.002 + 0.001652 * s + 0.0000083 * s * s) * 1e-3, rel=1e-15)


def _uniform_patch(n=16, dx=0.01):
    from beachslope_gb300 import abi, scene
    p = abi.default_params()
    p.h = 1.3 * dx
    p.dl = dx
    X0 = 4 * dx
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    x = X0 + (ii.ravel() + 0.5) * dx
    y = X0 + (jj.ravel() + 0.5) * dx
    st = scene._cat([scene._mk(x, y, np.full(n * n, 3), p.rho * dx * dx, p.rho, p.rho, dx * dx, -0.5)])
    scene._grid_for(p, X0 + (n + 4) * dx, X0 + (n + 4) * dx)
    return p, st


def test_lattice_interior_correction_is_identity(oracle):
    p, st = _uniform_patch()
    o = oracle.Oracle(p, st, None)
    o.stage("neighbour")
    s = o.get()
    c, *_ = o.neighbours(p.kmax)
    cx, cy = s["x"].mean(), s["y"].mean()
    inner = (np.abs(s["x"] - cx) < 3 * p.dl) & (np.abs(s["y"] - cy) < 3 * p.dl)
    assert inner.sum() > 10
    # a full symmetric lattice neighbourhood: 20 neighbours within 2.6 dx
    assert np.all(c[inner] == 20)
    np.testing.assert_allclose(s["coff"][inner][:, [0, 3]], 1.0, atol=0.05)
    np.testing.assert_allclose(s["coff"][inner][:, [1, 2]], 0.0, atol=1e-12)
    # interior particles are not free-surface particles
    assert not np.any(s["flags"][inner] & 1)


def test_porosity_limits(oracle):
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.02)
    o = oracle.Oracle(p, st, gr)
    o.stage("prime")
    s = o.get()
    f = s["tid"] == 3
    # no grains within 2h -> phi = 1; fully surrounded by grains -> phi = por
    assert s["porosity"][f].max() == 1.0
    assert s["porosity"][f].min() == pytest.approx(p.por, rel=1e-12)
    # walls keep porosity 1
    assert np.all(s["porosity"][~f] == 1.0)


def test_cell_binning_half_open(oracle):
    p, st = _uniform_patch(4)
    cw = 4 * p.h
    # particle exactly on a cell's right edge goes to the next cell (x < xright)
    st["x"][0] = 3 * cw
    o = oracle.Oracle(p, st, None)
    s = o.get()
    k = np.where(s["pid"] == st["pid"][0])[0][0]
    j = s["cell"][k] // p.celly + 1
    assert (j - 2) * cw <= 3 * cw < (j - 1) * cw
    assert j == 5


def _golden(name):
    return dict(np.load(os.path.join(GOLD, name)))


def _params_from(g):
    from beachslope_gb300 import abi
    p = abi.default_params()
    for k, v in g.items():
        if k.startswith("param_"):
            setattr(p, k[6:], v.item())
    return p


def _state_from(g, prefix="in_"):
    return {k[len(prefix):]: v for k, v in g.items() if k.startswith(prefix)}


def test_golden_beach_oracle_regression(oracle):
    g = _golden("beach_dx004.npz")
    p = _params_from(g)
    st = _state_from(g)
    gr = {k[6:]: v for k, v in g.items() if k.startswith("grain_")}
    o = oracle.Oracle(p, st, gr)
    o.stage("prime")
    s = o.get()
    np.testing.assert_array_equal(s["pid"], g["prime_pid"])
    np.testing.assert_allclose(s["porosity"], g["prime_porosity"], rtol=1e-12)
    np.testing.assert_allclose(s["coff"], g["prime_coff"], rtol=1e-9, atol=1e-12)
    c, idx, *_ = o.neighbours(p.kmax)
    np.testing.assert_array_equal(c, g["prime_nbr_count"])
    m = np.arange(p.kmax)[None, :] < c[:, None]
    np.testing.assert_array_equal(idx[m], g["prime_nbr_idx"])
    o.step(1)
    s = o.get()
    np.testing.assert_array_equal(s["pid"], g["step1_pid"])
    rel = np.linalg.norm(s["p"] - g["step1_p"]) / np.linalg.norm(g["step1_p"])
    assert rel < 1e-9
    np.testing.assert_allclose(s["x"], g["step1_x"], rtol=0, atol=1e-12)


def test_oracle_steps_stay_finite(oracle):
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.04)
    o = oracle.Oracle(p, st, gr)
    o.stage("prime")
    o.step(5)
    s = o.get()
    inf = o.info()
    assert np.all(np.isfinite(s["p"])) and np.all(np.isfinite(s["x"]))
    assert inf["err_bits"] == 0
    assert inf["ppe_relres"] <= p.ppe_tol


def test_ghost_row_leftover_entry_oracle(oracle):
    """isph.f90:125-128: a ghost row whose first neighbour is a lower-numbered
    fluid particle keeps val(1)=1.0 at col=row (an extra 1/dia on the diagonal
    after Jacobi scaling)."""
    from _scenes import ghost_row_scene
    p, st = ghost_row_scene()
    o = oracle.Oracle(p, st, None)
    for b in ("neighbour", "effpor", "int_vel", "ppe_assemble"):
        o.stage(b)
    d, off, rhs = o.matrix(p.kmax)
    s = o.get()
    c, idx, *_ = o.neighbours(p.kmax)
    q = np.where(d != 1.0)[0]
    assert len(q) > 0
    for r in q:
        j0 = idx[r, 0]
        assert s["tid"][r] == 2 and s["tid"][j0] == 3 and j0 < r


# ---------------------------------------------------------------- FGMRES
# fgmres (solver.f90:306-350) hands the system to MKL's dfgmres, which is
# closed and absent; the oracle restates restarted GMRES.  Pins: the 5x5
# known answer, and the defining property of the method -- after k columns
# of a cycle the iterate minimises ||b - A x|| over x0 + K_k(A, r0) -- checked
# against a dense least-squares solve, cycle by cycle across a restart.

def _nonsym(n, seed):
    rng = np.random.default_rng(seed)
    A = np.eye(n) * 4.0 + rng.standard_normal((n, n)) * (0.6 / np.sqrt(n))
    return A, rng.standard_normal(n)


def _csr(A):
    rows, cols = np.nonzero(A)
    ptr = np.zeros(A.shape[0] + 1, np.int64)
    np.add.at(ptr, rows + 1, 1)
    return np.cumsum(ptr), cols, A[rows, cols]


def _krylov_min(A, b, x0, k):
    r0 = b - A @ x0
    K = np.empty((len(b), k))
    v = r0 / np.linalg.norm(r0)
    for j in range(k):
        K[:, j] = v
        v = A @ v
        v = v / np.linalg.norm(v)
    Q, _ = np.linalg.qr(K)
    y, *_ = np.linalg.lstsq(A @ Q, r0, rcond=None)
    return x0 + Q @ y


def test_fgmres_known_answer(oracle):
    rc, x, it, rr = oracle.fgmres_csr(KAT_ROW, KAT_COL, KAT_VAL, KAT_B, np.ones(5), tol=1e-13, maxit=20,
                                      restart=5, rule=0)
    assert rc == 0 and it <= 5
    np.testing.assert_allclose(x, KAT_X, rtol=0, atol=1e-11)


@pytest.mark.parametrize("k", [1, 3, 6])
def test_fgmres_iterate_minimises_over_krylov_space(oracle, k):
    A, b = _nonsym(40, 3)
    ptr, col, val = _csr(A)
    x0 = np.full(40, 0.25)
    rc, x, it, rr = oracle.fgmres_csr(ptr, col, val, b, x0, tol=1e-300, maxit=k, restart=20, rule=0)
    assert it == k and rc != 0   # stopped by the column cap
    np.testing.assert_allclose(x, _krylov_min(A, b, x0, k), rtol=1e-10, atol=1e-12)


def test_fgmres_restart_cycles(oracle):
    A, b = _nonsym(40, 4)
    ptr, col, val = _csr(A)
    x0 = np.zeros(40)
    rc, x, it, rr = oracle.fgmres_csr(ptr, col, val, b, x0, tol=1e-300, maxit=7, restart=4, rule=0)
    assert it == 7
    x1 = _krylov_min(A, b, x0, 4)          # first cycle: 4 columns
    np.testing.assert_allclose(x, _krylov_min(A, b, x1, 3), rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("rule,tol", [(0, 1e-9), (2, 1e-3)])
def test_fgmres_stopping_rules(oracle, rule, tol):
    A, b = _nonsym(60, 5)
    ptr, col, val = _csr(A)
    x0 = np.ones(60)
    r0 = np.linalg.norm(b - A @ x0)
    rc, x, it, rr = oracle.fgmres_csr(ptr, col, val, b, x0, tol=tol, maxit=200, restart=150, rule=rule)
    assert rc == 0
    ref = tol * (np.linalg.norm(b) if rule == 0 else r0)
    res = np.linalg.norm(b - A @ x)
    assert res <= ref * (1 + 1e-6)
    # one column fewer does not meet the rule (the stop is the first column that does)
    rc2, x2, it2, _ = oracle.fgmres_csr(ptr, col, val, b, x0, tol=tol, maxit=it - 1, restart=150, rule=rule)
    assert rc2 != 0 and np.linalg.norm(b - A @ x2) > ref


def test_fgmres_scene_solve(oracle):
    """The reference's live PPE settings on a small beach scene (R0 rule,
    1e-3, restart and cap 150), from the warm start; the result agrees with
    a tight BiCGStab solve to the accuracy the rule implies."""
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.04)
    a = oracle.Oracle(p, st, gr)
    b = oracle.Oracle(p, st, gr)
    for o in (a, b):
        for name in ("neighbour", "effpor", "int_vel", "ppe_assemble"):
            o.stage(name)
    rc, it, rr = a.ppe_fgmres(1e-3, maxit=150, restart=150, rule=2)
    assert rc == 0 and 0 < it <= 150
    rc2, it2, rr2 = b.ppe_solve(1e-12, maxit=20000)
    assert rc2 == 0
    pa, pb = a.get()["p"], b.get()["p"]
    assert np.linalg.norm(pa - pb) / np.linalg.norm(pb) < 0.05


def test_step_runs_the_named_solver(oracle):
    """The oracle's step solves the PPE with the solver the parameters name
    (ppe_solver): FGMRES and BiCGStab steps to 1e-12 give the same state, and
    FGMRES's column count is what the step reports."""
    from beachslope_gb300 import abi, scene
    p, st, gr = scene.beach_scene(dx=0.04)
    p.ppe_tol = 1e-12
    p.ppe_maxit = 20000
    q = abi.Params.from_buffer_copy(p)
    q.ppe_solver = abi.SOLVER_FGMRES
    q.ppe_restart = 150
    q.ppe_maxit = 600
    a, b = oracle.Oracle(p, st, gr), oracle.Oracle(q, st, gr)
    for o in (a, b):
        o.stage("prime")
        o.step(2)
    ga, gb = a.get(), b.get()
    np.testing.assert_array_equal(ga["pid"], gb["pid"])
    assert np.linalg.norm(gb["p"] - ga["p"]) / np.linalg.norm(ga["p"]) < 1e-8
    assert np.max(np.abs(gb["x"] - ga["x"])) < 1e-12
    ia, ib = a.info(), b.info()
    assert ib["ppe_relres"] <= 1e-12 and ib["err_bits"] == 0
    assert ib["ppe_iters"] != ia["ppe_iters"]   # different methods, different counts


def test_oracle_reproducible_on_many_threads(oracle):
    """Two runs of the same steps on the default thread count give the same
    bits (the dot products add per-thread partial sums in a fixed order)."""
    from beachslope_gb300 import scene
    out = []
    for _ in range(2):
        p, st, gr = scene.beach_scene(dx=0.03)
        o = oracle.Oracle(p, st, gr)
        o.stage("prime")
        o.step(2)
        out.append(o.get())
    for f in ("p", "x", "y", "vx", "con"):
        np.testing.assert_array_equal(out[0][f], out[1][f], err_msg=f)
