"""The overlapped read-back (bs_download_async / bs_download_wait): the state
it returns is the state at the call, even when the next step is submitted
before the wait, and it equals the synchronous bs_download of the same state
bit for bit, for both precision forms and each scene of a batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "vx", "vy", "p", "mass", "rho", "oden", "ovol", "con", "tid", "pid", "flags")
SCENES = (0.02, 0.03)


def _ctx(api, precision):
    from beachslope_gb300 import scene
    made = [scene.beach_scene(dx=d, precision=precision) for d in SCENES]
    c = api.Context([m[0] for m in made], [m[1] for m in made], [m[2] for m in made], tuning="auto")
    c.prime()
    return c


@pytest.mark.parametrize("precision", [0, 1])
def test_async_readback_is_the_state_at_the_call(api, precision):
    ref = _ctx(api, precision)
    ref.step(2)
    want = [ref.download(s, full=False) for s in range(len(SCENES))]
    ref.step(1)
    want_next = [ref.download(s, full=False) for s in range(len(SCENES))]
    ref.close()
    for s in range(len(SCENES)):
        c = _ctx(api, precision)
        c.step(2)
        out = api.pinned_state(c.capacity_rows(s))
        h = c.download_async(s, out=out)
        c.step(1)   # submitted while the copy may still be running
        got = c.download_wait(h)
        for f in FIELDS:
            assert np.array_equal(got[f], want[s][f]), (s, f)
        now = c.download(s, full=False)
        for f in FIELDS:
            assert np.array_equal(now[f], want_next[s][f]), (s, f)
        c.close()


def test_async_readback_rejects_small_buffers(api):
    from beachslope_gb300.api import BeachSlopeError
    c = _ctx(api, 1)
    small = api.pinned_state(c.capacity_rows(0) - 256)
    with pytest.raises((BeachSlopeError, ValueError)):
        c.download_async(0, out=small)
    c.close()
