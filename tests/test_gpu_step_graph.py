"""The captured production step (one CUDA graph per step, the salinity
sub-steps and the Krylov loops as conditional nodes on the device) against
the eager step (the same stages launched one by one with the host's loops):
bit-identical fields and the same iteration counts, for both precision
forms, both Krylov methods, a batch of uneven scenes, and scenes whose
salinity takes several sub-steps per step (integrator.f90:941-949)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "vx", "vy", "p", "con", "rho", "mass", "pid")


def _pair(api, P, S, G, solver=None):
    a = api.Context(P, S, G, tuning="auto")
    b = api.Context(P, S, G, tuning="auto")
    for c in (a, b):
        if solver is not None:
            c.set_option("ppe_solver", solver)
    a.set_option("step_graph", 1)
    b.set_option("step_graph", 0)
    return a, b


def _same(a, b, nscenes):
    for s in range(nscenes):
        ga, gb = a.download(s), b.download(s)
        for f in FIELDS:
            assert np.array_equal(ga[f], gb[f]), (s, f)
        ia, ib = a.info(s), b.info(s)
        assert ia["ppe_iters"] == ib["ppe_iters"], (s, ia, ib)
        assert ia["solsteps"] == ib["solsteps"] and ia["err_bits"] == ib["err_bits"] == 0


@pytest.mark.parametrize("precision,solver", [(0, None), (1, None), (0, 0), (1, 0)])
def test_captured_step_equals_eager(api, precision, solver):
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.02, precision=precision)
    a, b = _pair(api, [p], [st], [gr], solver)
    for c in (a, b):
        c.prime()
        c.step(5)
    _same(a, b, 1)
    assert a.get_option("step_graph_steps") == 5 and b.get_option("step_graph_steps") == 0
    assert 1 <= a.get_option("step_graph_cached") <= 8
    assert a.launch_count() > 0


def test_captured_step_batch_and_several_salinity_substeps(api):
    """Three scenes of uneven size; two of them with a small turbulent
    Schmidt number, so the time-step rule gives them several salinity
    sub-steps per step (an odd and an even count among the scenes)."""
    from beachslope_gb300 import scene
    scenes = [scene.beach_scene(dx=d, A=a) for d, a in ((0.02, 0.05), (0.03, 0.08), (0.04, 0.03))]
    P = [s[0] for s in scenes]
    S = [s[1] for s in scenes]
    G = [s[2] for s in scenes]
    P[0].tschmidt = 1e-6   # dtsol = sig1 dl^2 / (1e-9 + numax / tschmidt) well below dt
    P[2].tschmidt = 4e-6
    a, b = _pair(api, P, S, G)
    for c in (a, b):
        c.prime()
        c.step(4)
    _same(a, b, 3)
    subs = [a.info(s)["solsteps"] for s in range(3)]
    assert max(subs) > 1, subs
    assert a.get_option("step_graph_steps") == 4


@pytest.mark.parametrize("precision", [0, 1])
def test_block_sizes_give_identical_steps(api, precision):
    """The autotuner's launch shapes (threads per block of the neighbour
    sweeps and of the particle-level multigrid kernels) change no result:
    every row is computed by the same code whatever block it falls in."""
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.02, precision=precision)
    ref = api.Context([p], [st], [gr], tuning="auto")
    ref.set_option("sweep_tpb", 256)
    ref.set_option("mg0_tpb", 256)
    ref.prime()
    ref.step(3)
    want = ref.download()
    for sw, mg in ((64, 128), (128, 64)):
        c = api.Context([p], [st], [gr], tuning="auto")
        c.set_option("sweep_tpb", sw)
        c.set_option("mg0_tpb", mg)
        assert c.get_option("sweep_tpb") == sw and c.get_option("mg0_tpb") == mg
        c.prime()
        c.step(3)
        got = c.download()
        for f in FIELDS:
            assert np.array_equal(got[f], want[f]), (sw, mg, f)
        assert c.info()["ppe_iters"] == ref.info()["ppe_iters"]
