"""Host logic of the request loop (beachslope_gb300/serve.py) on a fake
batched context: admission in arrival order into the smallest slot that
fits, later requests passing one that fits no free slot, slots freed on
completion, latencies on the step clock.  No GPU: the fake records the calls
the loop makes."""
import numpy as np


class _FakeCtx:
    def __init__(self, nslots):
        self.scene = [None] * nslots
        self.log = []
        self.t = 0

    def set_scene(self, s, params, state, grains):
        self.scene[s] = None if len(state["x"]) == 0 else state
        self.log.append(("set", s, len(state["x"])))

    def prime_scene(self, s):
        self.log.append(("prime", s))

    def step(self, n=1):
        self.t += n

    def info(self, s=0):
        return {"n": 0 if self.scene[s] is None else len(self.scene[s]["x"]), "t": self.t}

    def download(self, s=0, full=True):
        return self.scene[s]


def _server(caps, cell=(50, 20)):
    from beachslope_gb300 import abi, serve
    srv = serve.Server.__new__(serve.Server)
    t = abi.default_params()
    t.cellx, t.celly = cell
    srv.templates = [abi.Params.from_buffer_copy(t) for _ in caps]
    srv.caps = list(caps)
    srv.gcaps = [10 ** 6] * len(caps)
    srv.nslots = len(caps)
    srv.ctx = _FakeCtx(len(caps))
    return srv


def _req(rid, arrival, n, cell=(40, 10)):
    from beachslope_gb300 import abi, serve
    p = abi.default_params()
    p.cellx, p.celly = cell
    st = {"x": np.zeros(n)}
    return serve.Request(rid, float(arrival), p, st, {"x": np.zeros(0)})


def test_admission_order_slot_choice_and_latency():
    srv = _server([1000, 100])
    reqs = [_req(0, 0, 50), _req(1, 0, 500), _req(2, 1, 80), _req(3, 2, 20)]
    out = srv.run(reqs, steps=3, clock="steps")
    assert sorted(out) == [0, 1, 2, 3]
    sets = [e for e in srv.ctx.log if e[0] == "set" and e[2] > 0]
    # request 0 (50 rows) takes the small slot, request 1 (500) the large one
    assert sets[0] == ("set", 1, 50) and sets[1] == ("set", 0, 500)
    # both slots busy until step 3: requests 2 and 3 wait, then reuse them
    assert out[0]["admit"] == 0 and out[0]["done"] == 3 and out[0]["latency"] == 3
    assert out[2]["admit"] == 3 and out[3]["admit"] == 3
    assert out[2]["latency"] == out[2]["done"] - 1
    # every admission is primed alone, and every completion empties its slot
    assert [e for e in srv.ctx.log if e[0] == "prime"] == [("prime", s) for (_, s, _) in sets]
    assert sum(1 for e in srv.ctx.log if e[0] == "set" and e[2] == 0) == 4


def test_a_later_request_passes_one_that_fits_no_free_slot():
    srv = _server([1000, 100])
    reqs = [_req(0, 0, 900), _req(1, 0, 900), _req(2, 0, 60)]
    out = srv.run(reqs, steps=2, clock="steps")
    # request 1 needs the large slot, busy with request 0; request 2 fits the
    # small one and starts at once
    assert out[2]["admit"] == 0 and out[1]["admit"] == 2
    assert srv.nsteps == 4


def test_fits_checks_rows_grains_and_the_cell_grid():
    srv = _server([100])
    assert srv.fits(0, _req(0, 0, 100))
    assert not srv.fits(0, _req(0, 0, 101))
    assert not srv.fits(0, _req(0, 0, 10, cell=(60, 10)))   # grid wider than the slot's
    from beachslope_gb300 import serve
    t = srv.templates[0]
    assert serve.Server.slots_for_memory(t, 1000, 0, 1e12, 4000.0) == 64
    assert serve.Server.slots_for_memory(t, 1000, 0, 1.0, 4000.0) == 0


def _memory_server(budget, bytes_per_row=4000.0):
    """A server laid out by serve.Server.plan within `budget` bytes (two size
    classes, half of the budget each), on the fake context."""
    from beachslope_gb300 import abi, serve
    t = abi.default_params()
    t.cellx, t.celly = 50, 20
    classes = [(t, 1000, 0, 0.5, 8), (t, 100, 0, 0.5, 8)]
    counts, used = serve.Server.plan(classes, budget, bytes_per_row)
    caps = [1000] * counts[0] + [100] * counts[1]
    return _server(caps), counts, used


def test_slot_table_from_a_memory_budget():
    from beachslope_gb300 import abi, serve
    t = abi.default_params()
    t.cellx, t.celly = 50, 20
    per_big = serve.Server.slot_bytes(t, 1000, 0, 4000.0)
    per_small = serve.Server.slot_bytes(t, 100, 0, 4000.0)
    # room for one slot of each class: the budget binds
    srv, counts, used = _memory_server(2 * per_big + 0.5)
    assert counts == [1, int(per_big // per_small)] and used <= 2 * per_big + 0.5
    # a large budget: the concurrency limit binds
    _, counts, _ = _memory_server(1e15)
    assert counts == [8, 8]
    # a budget below one large slot leaves that class out
    _, counts, _ = _memory_server(1.5 * per_small / 0.5)
    assert counts[0] == 0 and counts[1] == 1


def test_a_small_memory_budget_forces_queueing_and_rejects_what_never_fits():
    """One slot per class fits the budget: requests of the large class queue
    behind each other; a request larger than every slot is rejected at once
    instead of waiting forever."""
    from beachslope_gb300 import abi, serve
    t = abi.default_params()
    t.cellx, t.celly = 50, 20
    budget = serve.Server.slot_bytes(t, 1000, 0, 4000.0) * 2 + 1.0
    classes = [(t, 1000, 0, 0.5, 8), (t, 100, 0, 0.5, 1)]
    counts, _ = serve.Server.plan(classes, budget, 4000.0)
    assert counts == [1, 1]
    srv = _server([1000, 100])
    reqs = [_req(0, 0, 800), _req(1, 0, 700), _req(2, 1, 900), _req(3, 1, 5000)]
    out = srv.run(reqs, steps=3, clock="steps")
    assert out[0]["admit"] == 0 and out[1]["admit"] == 3 and out[2]["admit"] == 6
    assert out[2]["latency"] == 9 - 1
    assert out[3]["error"] == "larger than every slot" and srv.rejected == [3]
