"""Host logic of the autotuner (beachslope_gb300/autotune.py) on a fake
context whose step time is a known function of the solver options: the
staged search finds the fastest configuration, skips candidates whose solves
report errors, restores the scene before every candidate and leaves the best
options set; the cache round-trips by size class."""
import json
import math


class _FakeCtx:
    nscenes = 1

    def __init__(self, cost, bad=()):
        self.opts = {}
        self.cost, self.bad = cost, bad
        self.uploads = 0

    def set_option(self, k, v):
        self.opts[k] = v

    def download(self, s=0):
        return {"x": [0.0]}

    def upload(self, s, st, gr=None):
        self.uploads += 1

    def clear_errors(self):
        pass

    def prime(self):
        pass

    def step(self, n=1):
        pass

    def sync(self):
        pass

    def record(self, slot):
        pass

    def elapsed_ms(self, a, b):
        return self.cost(self.opts) * 2   # _measure divides by its 2 steps

    def info(self, s=0):
        err = 1 if any(self.opts.get(k) == v for k, v in self.bad) else 0
        return {"err_bits": err, "ppe_iters": 10}


def test_staged_search_finds_the_fastest_and_skips_errors():
    from beachslope_gb300 import autotune

    def cost(o):
        c = 10.0
        c -= 2.0 if o.get("ppe_solver") == 1 and o.get("ppe_restart") == 50 else 0.0
        c -= 1.0 if o.get("mg_wlev") == 3 else 0.0
        c -= 0.5 if o.get("mg_omega") == 0.95 else 0.0
        c -= 3.0 if o.get("mg_cscale") == 1.7 else 0.0   # fastest, but its solves fail
        return c

    ctx = _FakeCtx(cost, bad=[("mg_cscale", 1.7)])
    best, ms, table = autotune.tune(ctx, [None], verbose=False)
    assert best["ppe_solver"] == 1 and best["ppe_restart"] == 50
    assert best["mg_wlev"] == 3 and best["mg_omega"] == 0.95 and best["mg_cscale"] != 1.7
    assert math.isclose(ms, 10.0 - 2.0 - 1.0 - 0.5)
    assert any(not row["ok"] for row in table)
    # every candidate started from the snapshot; the best options are left set
    assert ctx.uploads == len(table) + 1
    assert all(ctx.opts[k] == v for k, v in best.items())


def test_cache_round_trip(tmp_path, monkeypatch):
    from beachslope_gb300 import autotune
    monkeypatch.setattr(autotune, "CACHE", str(tmp_path / "tuning.json"))
    autotune.save(1, 700_000, {"mg_wlev": 2, "ppe_restart": 120, "ppe_solver": 1}, 21.0, "w")
    assert autotune.lookup(1, 712_460)["options"]["mg_wlev"] == 2   # same size class
    assert autotune.lookup(0, 712_460) is None                      # no entry of that precision
    assert autotune.key(1, 712_460) == "prec1_n4^10"
    # a size class without an entry falls back to the nearest single-scene class
    autotune.save(1, 180_000, {"mg_wlev": 1}, 7.0, "small")
    assert autotune.lookup(1, 3_000_000)["options"]["mg_wlev"] == 2
    assert autotune.lookup(1, 100_000)["options"]["mg_wlev"] == 1
    # a batch uses its own entry (size and scene-count class) when there is one
    assert autotune.key(1, 1_000_000, 64) == "prec1_n4^10_s4^3"
    assert autotune.lookup(1, 1_000_000, 64)["options"]["mg_wlev"] == 2
    autotune.save(1, 1_000_000, {"mg_wlev": 0}, 20.0, "batch", scenes=64)
    assert autotune.lookup(1, 1_000_000, 64)["options"]["mg_wlev"] == 0
    assert autotune.lookup(1, 712_460)["options"]["mg_wlev"] == 2
    ctx = _FakeCtx(lambda o: 1.0)
    autotune.apply(ctx, 1, 712_460)
    assert list(ctx.opts) == ["ppe_restart", "ppe_solver", "mg_wlev"]   # restart before the method
    assert json.load(open(autotune.CACHE))["prec1_n4^10"]["ms_per_step"] == 21.0
