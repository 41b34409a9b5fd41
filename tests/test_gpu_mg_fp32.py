"""The FP64 form with its multigrid preconditioner in FP32 (option mg_fp32):
the Krylov solve and its stopping test stay FP64, so the pressure is the
solution of the same FP64 system -- against the FP64 cycle, both solved to
1e-12, the pressure agrees to rounding -- and the captured step equals the
eager step bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx(api, mg_fp32, tol, step_graph=1):
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.01, precision=0)
    p.ppe_tol = tol
    p.ppe_maxit = 20000
    c = api.Context([p], [st], [gr], tuning="auto")
    c.set_option("mg_fp32", mg_fp32)
    c.set_option("step_graph", step_graph)
    assert c.get_option("mg_fp32") == mg_fp32
    c.prime()
    return c


def test_fp32_cycle_solves_the_same_fp64_system(api):
    a = _ctx(api, 0, 1e-12)
    b = _ctx(api, 1, 1e-12)
    for c in (a, b):
        c.step(1)
    ga, gb = a.download(), b.download()
    rel = np.linalg.norm(gb["p"] - ga["p"]) / np.linalg.norm(ga["p"])
    ia, ib = a.info(), b.info()
    print(f"p rel-L2 {rel:.2e}; columns FP64 cycle {ia['ppe_iters']}, FP32 cycle {ib['ppe_iters']}")
    assert ia["err_bits"] == 0 and ib["err_bits"] == 0
    assert ib["ppe_relres"] <= 1e-12 * 1.01
    assert np.array_equal(ga["pid"], gb["pid"])
    assert rel <= 1e-9, rel
    assert np.max(np.abs(gb["x"] - ga["x"])) <= 1e-13


def test_fp32_cycle_captured_equals_eager(api):
    a = _ctx(api, 1, 1e-8, step_graph=1)
    b = _ctx(api, 1, 1e-8, step_graph=0)
    for c in (a, b):
        c.step(3)
    ga, gb = a.download(), b.download()
    for f in ("x", "y", "vx", "vy", "p", "con"):
        assert np.array_equal(ga[f], gb[f]), f
    assert a.info()["ppe_iters"] == b.info()["ppe_iters"]
    assert a.get_option("step_graph_steps") == 3
