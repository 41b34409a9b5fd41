"""Request loop: a scene placed into a running batch (bs_set_scene +
bs_prime_scene) gives the same result as the same scene run alone, and the
scenes already running are not perturbed by it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _alone(api, req, steps):
    c = api.Context([req.params], [req.state], [req.grains])
    c.prime()
    c.step(steps)
    out = c.download()
    c.close()
    return out


def test_requests_same_alone_and_in_the_mix(api):
    from beachslope_gb300 import abi, scene, serve
    specs = [(0.03, 0.05, 0.0), (0.04, 0.08, 2.0), (0.025, 0.03, 3.0), (0.035, 0.06, 5.0)]
    reqs = []
    for k, (dx, A, t) in enumerate(specs):
        p, st, gr = scene.beach_scene(dx=dx, A=A, precision=abi.PREC_MIXED)
        reqs.append(serve.Request(k, t, p, st, gr))
    # two slots whose template is the finest scene: requests queue and
    # join while others are mid-run (arrivals counted in batched steps)
    tp, tst, tgr = scene.beach_scene(dx=0.025, precision=abi.PREC_MIXED)
    srv = serve.Server([(tp, len(tst["x"]) + 512, len(tgr["x"]) + 64)] * 2)
    steps = 4
    res = srv.run(reqs, steps, clock="steps")
    srv.close()
    assert sorted(res) == [0, 1, 2, 3]
    assert res[2]["admit"] > res[2]["arrival"]   # waited for a slot
    for req in reqs:
        a = _alone(api, req, steps)
        b = res[req.rid]["state"]
        assert res[req.rid]["info"]["err_bits"] == 0
        for f in ("x", "y", "vx", "vy", "p", "con"):
            assert np.array_equal(a[f], b[f]), (req.rid, f)


def test_set_scene_rejects_a_larger_grid(api):
    from beachslope_gb300 import abi, scene
    p, st, gr = scene.beach_scene(dx=0.04, precision=abi.PREC_MIXED)
    big = scene.beach_scene(dx=0.02, precision=abi.PREC_MIXED)
    c = api.Context([p], [st], [gr], capacity=[len(big[1]["x"])], grain_capacity=[len(big[2]["x"])])
    with pytest.raises(api.BeachSlopeError):
        c.set_scene(0, big[0], big[1], big[2])
    c.close()
