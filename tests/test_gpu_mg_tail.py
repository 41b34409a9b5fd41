"""The last two multigrid levels of a visit in one block per scene (option
mg_tail, k_mg_tail) against the same visit as separate launches (pre-sweep
and restriction, coarsest-level Jacobi, residual and second solve on a
W-cycle level, prolongation and post-sweep): bit-identical steps for both
precision forms, with the fused level on the V-cycle and on the W-cycle side
of the cycle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "vx", "vy", "p", "con", "rho", "pid")


def _run(api, precision, wlev, tail):
    from beachslope_gb300 import scene
    p, st, gr = scene.beach_scene(dx=0.01, precision=precision)
    c = api.Context([p], [st], [gr], tuning="auto")
    c.set_option("mg_sub", 0)
    c.set_option("mg_exact", 0)
    c.set_option("mg_wlev", wlev)
    c.set_option("mg_tail", tail)
    level = c.get_option("mg_tail_level")
    c.prime()
    c.step(3)
    out = c.download(full=False)
    info = c.info()
    c.close()
    return level, out, info


@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("wlev", [1, 2])
def test_tail_block_equals_separate_launches(api, precision, wlev):
    level, a, ia = _run(api, precision, wlev, 1)
    off, b, ib = _run(api, precision, wlev, 0)
    assert level >= 1 and off == 0
    for f in FIELDS:
        assert np.array_equal(a[f], b[f]), f
    assert ia["ppe_iters"] == ib["ppe_iters"] and ia["err_bits"] == 0
