"""Request loop: continuous batching of beach-slope scenes on one GPU.

The reference runs one scene per process and has no serving layer; this
module is the host side of the batched library for many independent
requests.  One batched context holds a fixed set of scene slots (row, grain
and cell-grid capacities from a template scene per slot, sized to the free
device memory when the server starts).  Requests arrive over time; a request
that fits a free slot is placed there with bs_set_scene and primed alone with
bs_prime_scene (the scenes already running are not touched), and from then on
every batched step -- one launch per stage for all slots -- advances it
together with the others.  When a request has done its steps its state is
read back and the slot is emptied (a scene with no particles costs nothing
in the row sweeps) for the next request.  Each request's result is the same
as running it alone: the batch computes every scene's reductions, multigrid
hierarchy and solver convergence on its own.

Latency of a request = completion time - arrival time (queueing included).

Admission by free device memory: `Server.for_memory` lays the slot table out
at start within a budget taken from the device's free memory (cudaMemGetInfo
through bs_device_memory): each size class gets its share of the budget, and
as many slots as that share holds at the measured device bytes per row of a
calibration context (capped by the class's concurrency limit).  A request
waits in the queue until a free slot of a class that holds it exists; one
larger than every slot is rejected at once.
"""
import collections
import time

import numpy as np

from . import abi, api

Request = collections.namedtuple("Request", "rid arrival params state grains")


class Server:
    """Slots of one batched context; `templates` = [(params, rows, grains)]:
    the largest scene each slot takes (its cell grid bounds the grids of the
    requests placed there)."""

    def __init__(self, templates, tuning=None):
        params = [abi.Params.from_buffer_copy(t[0]) for t in templates]
        caps = [int(t[1]) for t in templates]
        gcaps = [int(t[2]) for t in templates]
        self.nslots = len(params)
        self.templates = params
        self.caps, self.gcaps = caps, gcaps
        self.ctx = api.Context(params, [abi.empty_state() for _ in params], [None] * len(params),
                               capacity=caps, grain_capacity=gcaps, tuning=tuning)
        self.ctx.prime()

    @staticmethod
    def slot_bytes(template, rows, grains, bytes_per_row):
        """Device bytes one slot of `rows` rows reserves: the per-row arrays
        (particles, neighbour list, matrix, multigrid, Krylov basis) at the
        measured bytes per row, the grains and the per-cell arrays."""
        return rows * bytes_per_row + grains * 56.0 + template.cellx * template.celly * 120.0

    @staticmethod
    def slots_for_memory(template, rows, grains, budget_bytes, bytes_per_row, max_slots=64):
        """How many slots of one template fit in `budget_bytes` of device
        memory (0 when not even one does)."""
        per = Server.slot_bytes(template, rows, grains, bytes_per_row)
        return int(max(0, min(max_slots, budget_bytes // per)))

    @staticmethod
    def plan(classes, budget_bytes, bytes_per_row):
        """Slot table within a memory budget.  classes = [(template params,
        rows, grains, share of the budget, concurrency limit)]; returns the
        number of slots of each class and the bytes they reserve."""
        counts, used = [], 0.0
        for t, rows, grains, share, limit in classes:
            k = Server.slots_for_memory(t, rows, grains, share * budget_bytes, bytes_per_row, limit)
            counts.append(k)
            used += k * Server.slot_bytes(t, rows, grains, bytes_per_row)
        return counts, used

    @staticmethod
    def calibrate(params, state, grains, tuning=None):
        """Measured device bytes per row of a one-scene context holding
        `state` at 1.3x its rows, after prime and one production step (the
        Krylov basis is allocated at the first solve)."""
        rows = int(1.3 * len(state["x"]))
        ng = int(1.3 * len(grains["x"])) + 64 if grains is not None else 64
        c = api.Context([params], [state], [grains], capacity=[rows], grain_capacity=[ng], tuning=tuning)
        c.prime()
        c.step(1)
        b = c.device_bytes()
        c.close()
        return b / rows

    @classmethod
    def for_memory(cls, classes, bytes_per_row, budget_bytes=None, fraction=0.5, tuning=None):
        """A server whose slot table is laid out within `budget_bytes`
        (default: `fraction` of the device's free memory now)."""
        if budget_bytes is None:
            free, _ = api.device_memory()
            budget_bytes = fraction * free
        counts, used = cls.plan(classes, budget_bytes, bytes_per_row)
        if not any(counts):
            raise MemoryError("no slot fits the device memory budget")
        templates = []
        for (t, rows, grains, _, _), k in zip(classes, counts):
            templates += [(t, rows, grains)] * k
        srv = cls(templates, tuning=tuning)
        srv.budget_bytes, srv.planned_bytes, srv.bytes_per_row = budget_bytes, used, bytes_per_row
        srv.class_counts = counts
        return srv

    def fits(self, slot, req):
        t = self.templates[slot]
        ng = len(req.grains["x"]) if req.grains is not None else 0
        return (len(req.state["x"]) <= self.caps[slot] and ng <= self.gcaps[slot]
                and req.params.cellx <= t.cellx and req.params.celly <= t.celly)

    def run(self, requests, steps, clock="wall", on_done=None):
        """Serve `requests` (sorted by arrival), `steps` production steps
        each.  clock="wall": arrivals in seconds of wall time from the start;
        clock="steps": arrivals counted in batched steps (deterministic, for
        tests).  Returns {rid: result} with 'state', 'arrival', 'admit',
        'done', 'latency' (seconds, or steps with the step clock)."""
        reqs = sorted(requests, key=lambda r: r.arrival)
        ctx = self.ctx
        t0 = time.perf_counter()
        nsteps = 0

        def now():
            return nsteps if clock == "steps" else time.perf_counter() - t0

        queue = collections.deque()
        active = {}          # slot -> [request, steps left, admit time]
        free = list(range(self.nslots))
        out = {}
        i = 0
        self.step_ms = []
        self.rejected = []
        while i < len(reqs) or queue or active:
            tnow = now()
            while i < len(reqs) and reqs[i].arrival <= tnow:
                if any(self.fits(k, reqs[i]) for k in range(self.nslots)):
                    queue.append(reqs[i])
                else:   # no slot of the table can ever hold it
                    self.rejected.append(reqs[i].rid)
                    out[reqs[i].rid] = {"error": "larger than every slot", "arrival": reqs[i].arrival}
                i += 1
            # admission in arrival order; a request that fits no free slot
            # waits, and later requests that fit may pass it
            for req in list(queue):
                cands = [s for s in free if self.fits(s, req)]
                if not cands:
                    continue
                s = min(cands, key=lambda k: self.caps[k])
                ctx.set_scene(s, req.params, req.state, req.grains)
                ctx.prime_scene(s)
                free.remove(s)
                queue.remove(req)
                active[s] = [req, steps, now()]
            if not active:
                if clock == "steps":
                    nsteps = max(nsteps, int(np.ceil(reqs[i].arrival))) if i < len(reqs) else nsteps
                else:
                    time.sleep(max(0.0, min(0.01, reqs[i].arrival - now())) if i < len(reqs) else 0.0)
                continue
            ts = time.perf_counter()
            ctx.step(1)
            self.step_ms.append(1e3 * (time.perf_counter() - ts))
            nsteps += 1
            for s in list(active):
                a = active[s]
                a[1] -= 1
                if a[1] > 0:
                    continue
                req = a[0]
                info = ctx.info(s)
                res = {"state": ctx.download(s), "info": info, "arrival": req.arrival, "admit": a[2],
                       "done": now(), "n": len(req.state["x"])}
                res["latency"] = res["done"] - req.arrival
                out[req.rid] = res
                if on_done:
                    on_done(req, res)
                ctx.set_scene(s, self.templates[s], abi.empty_state(), None)
                del active[s]
                free.append(s)
        self.nsteps = nsteps
        return out

    def close(self):
        self.ctx.close()


def poisson_requests(n, rate, sizes=(5_000, 500_000), seed=20261203, precision=abi.PREC_MIXED):
    """n requests with Poisson arrivals (rate per second) and log-uniform
    particle counts in `sizes`; scene parameters as the batched beach scenes
    (slope 1:5..1:20, amplitude 0.02..0.10 m, porosity 0.3..0.5)."""
    from . import scene
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    counts = np.exp(rng.uniform(np.log(sizes[0]), np.log(sizes[1]), n))
    out = []
    for k in range(n):
        slope = 1.0 / rng.uniform(5.0, 20.0)
        A = rng.uniform(0.02, 0.10)
        por = rng.uniform(0.3, 0.5)
        dx = scene.dx_for_particles(counts[k])
        p, st, gr = scene.beach_scene(dx=dx, slope=slope, A=A, por=por, precision=precision)
        out.append(Request(k, float(t[k]), p, st, gr))
    return out
