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
    def slots_for_memory(template, rows, grains, budget_bytes, bytes_per_row=2600.0, max_slots=64):
        """How many slots of one template fit in `budget_bytes` of device
        memory (admission by free HBM when the pool is laid out)."""
        per = rows * bytes_per_row + grains * 40.0 + template.cellx * template.celly * 4 * 120.0
        return int(max(1, min(max_slots, budget_bytes // per)))

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
        while i < len(reqs) or queue or active:
            tnow = now()
            while i < len(reqs) and reqs[i].arrival <= tnow:
                queue.append(reqs[i])
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
