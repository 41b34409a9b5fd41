"""The mixed form of the WCSPH step (the continuity sweep on the FP32 pipe
from double-float copies of the cancelling fields, the other sweeps as in the
ISPH step) against the FP64 form from the same state: the continuity density
of one stage, then a few WCSPH steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def relmax(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _pair(api, form):
    from beachslope_gb300 import abi, scene
    out = []
    for prec in (abi.PREC_FP64, abi.PREC_MIXED):
        p, st, gr = scene.beach_scene(dx=0.02, A=0.06, wcsph=True, precision=prec)
        p.wc_form = form
        c = api.Context([p], [st], [gr])
        c.prime()
        c.stage("wcsph_pressure_to_density")
        out.append((c, p))
    return out


@pytest.mark.parametrize("form", [0, 1])
def test_mixed_continuity_against_fp64(api, form):
    (a, p), (b, _) = _pair(api, form)
    for c in (a, b):
        c.stage("wcsph_continuity")
        c.stage("wcsph_update_density")
    ga, gb = a.download(), b.download()
    fl = ga["tid"] == 3
    e = relmax(gb["rho"][fl] - p.rho, ga["rho"][fl] - p.rho)
    print(f"form {form}: continuity density change, mixed vs FP64 max rel {e:.2e}")
    assert e < 1e-5, e
    assert b.info()["err_bits"] == 0


def test_mixed_wcsph_steps_against_fp64(api):
    (a, p), (b, _) = _pair(api, 1)
    for k in range(4):
        a.wcsph_step(1)
        b.wcsph_step(1)
    ga, gb = a.download(), b.download()
    oa, ob = np.argsort(ga["pid"]), np.argsort(gb["pid"])
    assert np.array_equal(ga["pid"][oa], gb["pid"][ob])
    erho = relmax(gb["rho"][ob] - p.rho, ga["rho"][oa] - p.rho)
    ep = relmax(gb["p"][ob], ga["p"][oa])
    ev = relmax(gb["vx"][ob], ga["vx"][oa])
    print(f"4 WCSPH steps, mixed vs FP64: rho change {erho:.2e}, p {ep:.2e}, vx {ev:.2e}")
    assert erho < 1e-4 and ep < 1e-5 and ev < 1e-5
    assert b.info()["err_bits"] == 0
