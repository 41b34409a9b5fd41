"""Per-step pressure of the mixed form against the FP64 drop-in, scene by
scene, in a batch of coarse beach scenes (dx 12-20 mm: few particles per
wave height, wall rows a large share, where the mixed form's error is
largest).  The batch runs 100 mixed steps; from that common state each form
takes one step with the PPE solved to 1e-12 in both, so the difference is
the mixed arithmetic's and not the solver tolerance's.  Bar: relative L2
of p <= 1e-6 for every scene."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ("x", "y", "vx", "vy", "p", "mass", "rho", "oden", "ovol", "con", "tid", "pid", "flags")


def test_batch_step_pressure_per_scene(api):
    from beachslope_gb300 import abi, scene
    sc = scene.batch_scenes(12, precision=abi.PREC_MIXED, dx_range=(0.012, 0.02))
    P, S, G = [q[0] for q in sc], [q[1] for q in sc], [q[2] for q in sc]
    c = api.Context(P, S, G, tuning="auto")
    c.prime()
    c.step(100)
    st = [{k: c.download(s, full=False)[k].copy() for k in KEYS} for s in range(len(P))]
    assert c.info()["err_bits"] == 0
    c.close()

    def one(prec):
        Q = [abi.Params.from_buffer_copy(p) for p in P]
        for q in Q:
            q.precision = prec
            q.ppe_tol = 1e-12
            q.ppe_maxit = 20000
        cc = api.Context(Q, st, G, tuning="auto")
        cc.prime()
        cc.step(1)
        out = [cc.download(s, full=False) for s in range(len(Q))]
        info = [cc.info(s) for s in range(len(Q))]
        cc.close()
        return out, info

    m, im = one(abi.PREC_MIXED)
    f, iff = one(abi.PREC_FP64)
    errs = []
    for s in range(len(P)):
        a, b = m[s], f[s]
        oa, ob = np.argsort(a["pid"]), np.argsort(b["pid"])
        assert np.array_equal(a["pid"][oa], b["pid"][ob])
        assert im[s]["err_bits"] == 0 and iff[s]["err_bits"] == 0
        assert im[s]["ppe_relres"] <= 1e-11 and iff[s]["ppe_relres"] <= 1e-11
        errs.append(float(np.linalg.norm(a["p"][oa] - b["p"][ob]) / np.linalg.norm(b["p"])))
    print("per-scene p rel-L2, mixed vs FP64 at 1e-12: max %.2e median %.2e (n %s)"
          % (max(errs), float(np.median(errs)), [len(x["p"]) for x in f]))
    assert max(errs) <= 1e-6, errs
