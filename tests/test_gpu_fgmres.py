"""GPU tests of the FGMRES option (ppe_solver = BS_SOLVER_FGMRES): the
Krylov method of the reference's live PPE solve (fgmres, solver.f90:306-350).

Against the oracle's restated GMRES on the same system: the same number of
Arnoldi columns, and iterates equal to rel-L2 1e-9 (the GPU orthogonalises by
classical Gram-Schmidt applied twice, the oracle by modified Gram-Schmidt;
both give the Krylov minimiser to round-off).  Preconditioned (multigrid)
solves are checked against a tight BiCGStab solve of the same system.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KAT_ROW = np.array([1, 4, 6, 8, 11, 14]) - 1
KAT_COL = np.array([1, 3, 4, 2, 4, 1, 3, 2, 3, 4, 1, 2, 5]) - 1


def relL2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _banded(n, seed):
    """Non-symmetric, diagonally dominant, 9 entries per row."""
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for i in range(n):
        for d in (-40, -7, -3, -1, 0, 1, 2, 9, 31):
            j = i + d
            if 0 <= j < n:
                rows.append(i)
                cols.append(j)
                vals.append(4.0 if d == 0 else rng.uniform(-0.5, 0.4))
    import scipy.sparse as sp
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    return A, rng.standard_normal(n)


def test_fgmres_known_answer_gpu(api):
    rc, x, it, rr = api.fgmres_csr(KAT_ROW, KAT_COL, np.ones(13), [8.0, 6.0, 4.0, 9.0, 8.0], np.ones(5),
                                   tol=1e-13, maxit=20, restart=5, rule=0)
    assert rc == 0 and it <= 5
    np.testing.assert_allclose(x, [1, 2, 3, 4, 5], rtol=0, atol=1e-10)


@pytest.mark.parametrize("n,restart,tol,rule,maxit", [
    (3000, 30, 1e-10, 0, 2000),     # restarted, relative to ||b||
    (3000, 150, 1e-3, 2, 150),      # the reference's settings
    (5000, 8, 1e-300, 0, 21),       # column cap inside the third cycle
])
def test_fgmres_csr_matches_oracle(api, oracle, n, restart, tol, rule, maxit):
    A, b = _banded(n, n + restart)
    x0 = np.full(n, 0.1)
    rg, xg, ig, rrg = api.fgmres_csr(A.indptr, A.indices, A.data, b, x0, tol=tol, maxit=maxit, restart=restart,
                                     rule=rule)
    ro, xo, io, rro = oracle.fgmres_csr(A.indptr, A.indices, A.data, b, x0, tol=tol, maxit=maxit,
                                        restart=restart, rule=rule)
    assert (rg == 0) == (ro == 0)
    assert ig == io
    assert relL2(xg, xo) < 1e-9
    assert abs(rrg - rro) <= 1e-6 * rro + 1e-15


def _assembled(api, oracle, p, st, gr):
    ctx = api.Context([p], [st], [gr])
    o = oracle.Oracle(p, st, gr)
    for a, b in (("search", "neighbour"), ("porosity", "effpor"), ("int_vel", "int_vel"),
                 ("ppe_assemble", "ppe_assemble")):
        ctx.stage(a)
        o.stage(b)
    return ctx, o


def test_fgmres_scene_reference_settings(api, oracle):
    """Unpreconditioned FGMRES, ||r|| <= 1e-3 ||r0||, restart = cap = 150, from
    the warm start (the previous pressure): the GPU and the oracle take the
    same number of columns and agree on the pressure."""
    from beachslope_gb300 import abi, scene
    p, st, gr = scene.beach_scene(dx=0.02)
    p.ppe_solver = abi.SOLVER_FGMRES
    p.ppe_restart = 150
    p.ppe_maxit = 150
    p.ppe_precond = 0
    p.ppe_stop = abi.STOP_R0
    p.ppe_tol = 1e-3
    ctx, o = _assembled(api, oracle, p, st, gr)
    ctx.ppe_solve()
    rc, it, rr = o.ppe_fgmres(1e-3, maxit=150, restart=150, rule=abi.STOP_R0)
    assert rc == 0
    info = ctx.info()
    assert info["ppe_iters"] == it and info["err_bits"] == 0
    g, ref = ctx.download(), o.get()
    np.testing.assert_array_equal(g["pid"], ref["pid"])
    assert relL2(g["p"], ref["p"]) < 1e-8


@pytest.mark.parametrize("precision", [0, 1])
def test_fgmres_multigrid_matches_bicgstab(api, precision):
    """FGMRES right-preconditioned by the multigrid cycle (FP64, or FP32 in
    the mixed form) to ||r||/||b|| <= 1e-12: the pressure agrees with the
    BiCGStab solve of the same system."""
    from beachslope_gb300 import abi, scene
    p, st, gr = scene.beach_scene(dx=0.01, precision=precision)
    p.ppe_tol = 1e-12
    p.ppe_maxit = 5000
    q = abi.Params.from_buffer_copy(p)
    q.ppe_solver = abi.SOLVER_FGMRES
    q.ppe_restart = 30
    a = api.Context([p], [st], [gr])
    b = api.Context([q], [st], [gr])
    for c in (a, b):
        for name in ("search", "porosity", "int_vel", "ppe_assemble", "ppe_solve"):
            c.stage(name)
    ia, ib = a.info(), b.info()
    assert ia["err_bits"] == 0 and ib["err_bits"] == 0 and ib["ppe_relres"] <= 1e-12
    assert ib["ppe_iters"] > 0
    assert relL2(b.download()["p"], a.download()["p"]) < 1e-6


def test_fgmres_batched_equal_alone(api):
    """Three scenes in one batch (lock-step cycles, per-scene reductions)
    end bit-identical to each scene solved alone, over steps."""
    from beachslope_gb300 import abi, scene
    scenes = [scene.beach_scene(dx=d, A=a) for d, a in ((0.03, 0.05), (0.04, 0.08), (0.05, 0.03))]
    P = [s[0] for s in scenes]
    for p in P:
        p.ppe_solver = abi.SOLVER_FGMRES
        p.ppe_restart = 20
    S = [s[1] for s in scenes]
    G = [s[2] for s in scenes]
    batch = api.Context(P, S, G)
    batch.prime()
    batch.step(3)
    for k in range(3):
        alone = api.Context([P[k]], [S[k]], [G[k]])
        alone.prime()
        alone.step(3)
        x, y = alone.download(), batch.download(k)
        for f in ("x", "y", "vx", "vy", "p", "con"):
            assert np.array_equal(x[f], y[f]), f
        assert alone.info()["ppe_iters"] == batch.info(k)["ppe_iters"]


def test_fgmres_steps_match_bicgstab(api):
    """Production steps with the FGMRES option (multigrid, 1e-12) against
    the BiCGStab steps from the same state."""
    from beachslope_gb300 import abi, scene
    p, st, gr = scene.beach_scene(dx=0.02)
    p.ppe_tol = 1e-12
    p.ppe_maxit = 5000
    q = abi.Params.from_buffer_copy(p)
    q.ppe_solver = abi.SOLVER_FGMRES
    q.ppe_restart = 40
    a = api.Context([p], [st], [gr])
    b = api.Context([q], [st], [gr])
    for c in (a, b):
        c.prime()
        c.step(2)
    ga, gb = a.download(), b.download()
    oa, ob = np.argsort(ga["pid"]), np.argsort(gb["pid"])
    np.testing.assert_array_equal(ga["pid"][oa], gb["pid"][ob])
    assert relL2(gb["p"][ob], ga["p"][oa]) < 1e-6
    assert b.info()["err_bits"] == 0


def test_fgmres_options(api):
    from beachslope_gb300 import abi, scene
    p, st, gr = scene.beach_scene(dx=0.04)
    ctx = api.Context([p], [st], [gr])
    ctx.set_option("ppe_solver", abi.SOLVER_FGMRES)
    ctx.set_option("ppe_restart", 12)
    assert ctx.get_option("ppe_solver") == abi.SOLVER_FGMRES and ctx.get_option("ppe_restart") == 12
    ctx.prime()
    ctx.step(1)
    assert ctx.info()["err_bits"] == 0
    with pytest.raises(Exception):
        ctx.set_option("ppe_restart", 151)


@pytest.mark.parametrize("tol", [1e-8, 1e-12])
def test_fgmres_double_float_basis(api, tol):
    """The mixed solve's double-float basis (fg_df = 1: (hi, lo) FP32 pairs,
    dots and projection on the FP32 pipe) against the FP64 basis (fg_df = 0)
    on the same system: the same column count within one, pressures within
    1e-6 (tolerance 1e-8) and 1e-9 (tolerance 1e-12)."""
    from beachslope_gb300 import abi, scene
    p, st, gr = scene.beach_scene(dx=0.01, precision=abi.PREC_MIXED)
    p.ppe_solver = abi.SOLVER_FGMRES
    p.ppe_restart = 40
    p.ppe_tol = tol
    p.ppe_maxit = 400
    res = []
    for df in (0, 1):
        c = api.Context([p], [st], [gr])
        c.set_option("fg_df", df)
        assert c.get_option("fg_df") == df
        for name in ("search", "porosity", "int_vel", "ppe_assemble", "ppe_solve"):
            c.stage(name)
        res.append((c.info(), c.download()["p"]))
    (i0, p0), (i1, p1) = res
    assert i0["err_bits"] == 0 and i1["err_bits"] == 0
    assert i1["ppe_relres"] <= tol and abs(i1["ppe_iters"] - i0["ppe_iters"]) <= 1
    assert relL2(p1, p0) < (1e-6 if tol > 1e-10 else 1e-9)
