"""The mixed search's stored pair values against the FP64 search's on the
same positions (the primed state of the dx = 10 mm beach, 13 k particles).

The mixed search works on the FP32 pipe from double-float positions: r by a
double-float Newton step, the kernel gradient F(r) (x_i - x_j) in
double-float arithmetic with one FP32 scale per scene, each value rounded to
FP32 once.  So each stored value is the FP32 rounding of the FP64 value up
to ties: at most one FP32 ulp apart everywhere, and equal for all but a few
pairs in 10^4.  The gradient-correction matrix is summed from those stored
values with exact products, so it differs from the FP64 one by the FP32
rounding of the gradients: within 1e-6 relative, with the same rows
falling back to the identity (|det| < 1e-5)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _within_one_ulp(a, b64):
    """a (FP32 values widened to double) against b64 rounded to FP32: the
    largest distance in units of b's FP32 spacing, and the share of
    values that differ."""
    b32 = b64.astype(np.float32)
    d = np.abs(a - b32.astype(np.float64))
    sp = np.spacing(np.abs(b32)).astype(np.float64)
    return float(np.max(d / sp)), float(np.mean(a != b32.astype(np.float64)))


def test_mixed_pair_values_round_once(api):
    from beachslope_gb300 import abi, scene
    p, st, gr = scene.beach_scene(dx=0.01)
    pm = abi.Params.from_buffer_copy(p)
    pm.precision = abi.PREC_MIXED
    a = api.Context([p], [st], [gr])
    b = api.Context([pm], [st], [gr])
    a.prime()
    b.prime()
    ca, ia, da, kxa, kya = a.neighbours()
    cb, ib, db, kxb, kyb = b.neighbours()
    np.testing.assert_array_equal(ca, cb)
    m = np.arange(p.kmax)[None, :] < ca[:, None]
    np.testing.assert_array_equal(ia[m], ib[m])
    for name, mixed, fp64 in (("r", db, da), ("grad_x W", kxb, kxa), ("grad_y W", kyb, kya)):
        ulps, share = _within_one_ulp(mixed[m], fp64[m])
        print(f"{name}: {int(m.sum())} pairs, max {ulps:.2f} FP32 ulp, {share:.2e} differ")
        assert ulps <= 1.0, (name, ulps)
        assert share <= 1e-4, (name, share)
    ga, gb = a.download(), b.download()
    np.testing.assert_array_equal(ga["pid"], gb["pid"])
    fl = ga["tid"] == 3
    Ca, Cb = ga["coff"].reshape(-1, 4)[fl], gb["coff"].reshape(-1, 4)[fl]
    ident = np.all(Ca == np.array([1.0, 0.0, 0.0, 1.0]), axis=1)
    np.testing.assert_array_equal(ident, np.all(Cb == np.array([1.0, 0.0, 0.0, 1.0]), axis=1))
    rel = np.max(np.abs(Cb - Ca)) / np.max(np.abs(Ca))
    print(f"correction matrix: {int(fl.sum())} fluid rows, max difference {rel:.2e} of max |C|")
    assert rel <= 1e-6, rel
    assert a.info()["err_bits"] == 0 and b.info()["err_bits"] == 0
