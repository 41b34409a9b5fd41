"""Benchmark: particle-steps/s of the ISPH production step on one GB300.

    python bench.py [--gpus N --steps K --warmup W] [--workload W] [--precision P]
    python bench.py --impl reference ...     # the reference's CPU path (oracle port)

One "step" is one production time step (main.f90:199-272) of every scene of
the workload, with inputs already resident in HBM.  The default workload is
the refined solitary-wave beach scene (dx = 1.25 mm, h = 1.3 dx, dt = 1e-4 s,
BiCGStab to relative residual 1e-8).  Inputs are synthetic (seeded scene
generator); the state (> 100 MB) is larger than half of L2 and the step
streams all of it many times, so no L2 flush is needed between steps.

Prints ONE JSON line on rank 0.  N > 1 runs N independent replicas (one
process per GPU, no collective on the data path): value = all ranks'
particle-steps / max-over-ranks time.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

ge.load_package()

METRIC = "particle-steps/s (mixed vs FP64, same GPU, ≤1e-6 rel p); p99 scene latency"
UNIT = "particle-steps/s"

WORKLOADS = {
    "beach_dx0.00125": "solitary wave A=0.06 m on a 1:10 porous beach, dx=1.25 mm (~0.7M particles)",
    "beach_dx0.0025": "solitary wave A=0.06 m on a 1:10 porous beach, dx=2.5 mm (~0.18M particles)",
    "beach_dx0.01": "solitary wave A=0.06 m on a 1:10 porous beach, dx=10 mm (~15k particles)",
}


def build_workload(name, precision):
    from beachslope_gb300 import abi, scene
    dx = float(name.split("dx")[1])
    p, st, gr = scene.beach_scene(dx=dx, precision=precision)
    return [p], [st], [gr]


# ------------------------------------------------------------------ ranks
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.dist = dist

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def allreduce(self, v, op="max"):
        if self.world == 1:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX if op == "max" else self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


def aggregate(D, n_particles, steps, ms):
    """Whole-job throughput of N replicas: every rank's particle-steps over
    the slowest rank's time (value, max ms)."""
    ms_max = D.allreduce(ms, "max")
    parts = D.allreduce(n_particles, "sum")
    return parts * steps / (ms_max / 1e3), ms_max


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [c.strip() for c in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].strip() == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ------------------------------------------------------------- our arm
# Kernels bracketed by CUDA events during the timed region (the candidates for
# the dominant kernel).
TIMED_KERNELS = ("search_effpor", "bicg_it1_spmv", "bicg_it2_spmv", "mg_l0_down", "mg_l0_up",
                 "fg_arnoldi_spmv", "fg_project")
# DRAM bytes per launch measured by ncu over the algorithmic bytes of the same
# launch (0.18 M-particle beach, mixed; profiles/*_beach_dx0.0025_mixed.md);
# the traffic grows with the nonzeros and rows, so the ratio scales it to the
# bench's workload.  k_it2_64 has k_it1_64's access pattern.
TRAFFIC_RATIO = {"search_effpor": 0.46, "bicg_it1_spmv": 0.99, "bicg_it2_spmv": 0.99,
                 "mg_l0_down": 0.98, "mg_l0_up": 0.93, "fg_arnoldi_spmv": 0.99, "fg_project": 0.97}


def fg_columns(iters, restart):
    """Sum over the Arnoldi columns of one FGMRES solve of (j+1), the basis
    vectors column j reads (cycles of `restart` columns)."""
    tot, left = 0, int(iters)
    while left > 0:
        k = min(left, restart)
        tot += k * (k + 1) // 2
        left -= k
    return tot


def algorithmic_bytes(ctx, kernel, precision, basis_reads=None):
    """Compulsory HBM bytes of one launch over all scenes (neighbour-vector
    gathers counted as on-chip hits; every other operand read or written once).
    w = width of the per-pair and matrix values (8 FP64, 4 mixed).  For the
    FGMRES column kernels, basis_reads = the mean number of basis vectors a
    launch reads (j+1 at column j)."""
    w = 4 if precision == "mixed" else 8
    tot = 0.0
    for s in range(ctx.nscenes):
        c = ctx.neighbour_counts(s)
        nnz, n = float(c.sum()), float(len(c))
        if kernel == "fg_arnoldi_spmv":
            # SpMV (FP64 values + index; diag, count, input, output) + v_j + Z_j write + basis reads
            tot += nnz * (8 + 4) + n * (8 + 4 + 8 + 8) + n * (8 + 8) + basis_reads * n * 8
        elif kernel == "fg_project":
            tot += n * (8 + 8) + basis_reads * n * 8
        elif kernel in ("bicg_it1_spmv", "bicg_it2_spmv"):
            # values (FP64) + column index per nonzero; diag, count, input, output, dot operand per row
            tot += nnz * (8 + 4) + n * (8 + 4 + 8 + 8 + 8)
        elif kernel == "mg_l0_down":
            tot += nnz * (w + 4) + n * (8 + 4 + w + 8) + n / 27.0 * w
        elif kernel == "mg_l0_up":
            tot += nnz * (w + 4) + n * (8 + 4 + w + 8 + 4 + 8)
        elif kernel == "search_effpor":
            # own position, vol, flags, cell; list (index + dist, 1/(r2+lam), gradW x,y);
            # coff, gradvx, flags, count; effpor reads/writes
            tot += n * (16 + 8 + 2 + 4) + nnz * (4 + 4 * w) + n * (32 + 8 + 1 + 4) + n * (32 + 40)
    return tot


def fp64_flops(ctx, kernel, basis_reads, df=False):
    """Algorithmic FP64 operations of one launch (FMA = 2) for the FGMRES
    column kernels: SpMV (diagonal + nonzeros), two dots per basis vector
    (pass 1), one update per basis vector and the norm (pass 2).  In the
    mixed form (df) the basis work and the off-diagonal SpMV products run in
    double-float on the FP32 pipe: FP64 is left with the diagonal product and
    u.u (pass 1) and the final subtraction and scaling of each row (pass 2)."""
    tot = 0.0
    for s in range(ctx.nscenes):
        c = ctx.neighbour_counts(s)
        nnz, n = float(c.sum()), float(len(c))
        if kernel == "fg_arnoldi_spmv":
            tot += 4 * n if df else 2 * nnz + 2 * n + 4 * basis_reads * n
        elif kernel == "fg_project":
            tot += 2 * n if df else 2 * n + 2 * basis_reads * n
    return tot or None


def run_ours(args, D):
    from beachslope_gb300 import abi, api
    api.set_device(D.local)
    prec = abi.PREC_MIXED if args.precision == "mixed" else abi.PREC_FP64
    P, S, G = build_workload(args.workload, prec)
    n_particles = sum(len(s["x"]) for s in S)
    ctx = api.Context(P, S, G, tuning="auto")
    ctx.prime()
    for _ in range(args.warmup):
        ctx.step(1)
    ctx.sync()
    clocks = ClockSampler(D.local)
    D.barrier()
    ctx.sync()
    clocks.start()
    l0 = ctx.launch_count()
    ctx.record(0)
    ctx.step(args.steps)
    ctx.record(1)
    ms = ctx.elapsed_ms(0, 1)
    l1 = ctx.launch_count()
    ck = clocks.stop()
    D.barrier()
    # second timed pass of the same K steps with CUDA events around each launch
    # of the candidate kernels (graphs are off while events are on): the
    # per-launch durations of the roofline
    ids = ctx.kernel_ids()
    ctx.kernel_timing(sum(1 << ids[k] for k in TIMED_KERNELS if k in ids))
    ms_timed, fg_reads, fg_launches = 0.0, 0, 0
    restart = int(ctx.get_option("ppe_restart"))
    for _ in range(args.steps):   # one step at a time: each step's FGMRES column count
        ctx.record(2)
        ctx.step(1)
        ctx.record(3)
        ms_timed += ctx.elapsed_ms(2, 3)
        for s in range(ctx.nscenes):
            it = ctx.info(s)["ppe_iters"]
            fg_reads += fg_columns(it, restart)
            fg_launches += it
    kt = ctx.kernel_times()
    ctx.kernel_timing(0)
    value, ms_max = aggregate(D, n_particles, args.steps, ms)
    info = [ctx.info(s) for s in range(ctx.nscenes)]
    out = {
        "value": value,
        "ms_per_step": ms_max / args.steps,
        "particles": n_particles,
        "gpu_launches": int(l1 - l0),
        "clocks": ck,
        "ppe_iters_last": float(np.mean([i["ppe_iters"] for i in info])),
        "ppe_relres_last": max(i["ppe_relres"] for i in info),
        "err_bits": int(np.bitwise_or.reduce([i["err_bits"] for i in info])),
        "tuning": ctx.tuning["options"] if ctx.tuning else None,
    }
    # roofline of the dominant kernel (largest event-timed total)
    cands = [(k, v[0], v[1]) for k, v in kt.items() if k in TIMED_KERNELS and v[0]]
    if cands:
        name, cnt, tms = max(cands, key=lambda t: t[2])
        alg = algorithmic_bytes(ctx, name, args.precision, basis_reads=fg_reads / max(fg_launches, 1))
        avg_s = tms / cnt / 1e3
        pk, src = peaks()
        achieved = alg / avg_s / 1e9
        out["roofline"] = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": pk,
                           "peak_source": src, "unit": "GB/s", "frac": round(achieved / pk, 4),
                           "traffic": (round(TRAFFIC_RATIO[name] * alg) if args.precision == "mixed" else None),
                           "traffic_source": "ncu dram__bytes_read+write on the 0.18 M-particle case, scaled",
                           "algorithmic_bytes_per_launch": alg,
                           "avg_launch_us": round(avg_s * 1e6, 2), "launches": cnt,
                           "basis_vectors_per_launch": (round(fg_reads / max(fg_launches, 1), 2)
                                                        if name.startswith("fg_") else None),
                           "share_of_step": round(tms / ms_timed, 3),
                           "note": "durations from a second pass of the same steps with per-launch events",
                           "timed_kernels": {k: {"launches": v[0], "ms": round(v[1], 3)} for k, v in kt.items()}}
        df = (args.precision == "mixed" and int(ctx.get_option("ppe_solver")) == abi.SOLVER_FGMRES
              and int(ctx.get_option("fg_df")) == 1 and P[0].ppe_precond == 1)
        fl = fp64_flops(ctx, name, fg_reads / max(fg_launches, 1), df)
        if fl:
            out["roofline"]["fp64"] = {"flops_per_launch": round(fl), "achieved_tflops": round(fl / avg_s / 1e12, 3),
                                       "nominal_peak_tflops": 1.25,
                                       "frac": round(fl / avg_s / 1e12 / 1.25, 3)}
            if df:
                out["roofline"]["fp64"]["note"] = ("basis dots, projection and off-diagonal SpMV in "
                                                   "double-float on the FP32 pipe")
    state = ctx.download(0)
    ctx.close()
    if not args.no_e2e:
        out["e2e"] = run_e2e(args, D, P, S, G)
    if args.precision == "mixed" and not args.no_fp64:
        out["fp64"] = run_fp64_and_accuracy(args, P, S, G, state)
    return out


def run_fp64_and_accuracy(args, P, S, G, state):
    """The plain FP64 path on the same workload (same steps), and the per-step
    pressure error of the mixed form against it from one common state:
    both restart from the mixed run's final state and take one step, once at
    the configured PPE tolerance and once at 1e-12 (which isolates the
    precision of the sweeps and V-cycle from the solver tolerance)."""
    from beachslope_gb300 import abi, api
    P64 = [abi.Params.from_buffer_copy(p) for p in P]
    for p in P64:
        p.precision = abi.PREC_FP64
    c = api.Context(P64, S, G, tuning="auto")
    c.prime()
    for _ in range(args.warmup):
        c.step(1)
    c.sync()
    c.record(0)
    c.step(args.steps)
    c.record(1)
    ms = c.elapsed_ms(0, 1)
    n = sum(len(s["x"]) for s in S)
    res = {"value": n * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
           "ppe_iters_last": c.info(0)["ppe_iters"]}
    c.close()
    keys = ["x", "y", "vx", "vy", "p", "mass", "rho", "oden", "ovol", "con", "tid", "pid", "flags"]
    st = {k: state[k] for k in keys}
    def one_step(prec, tol, precond=1):
        q = abi.Params.from_buffer_copy(P[0])
        q.precision = prec
        q.ppe_tol = tol
        q.ppe_maxit = 20000
        q.ppe_precond = precond
        cc = api.Context([q], [st], [G[0]], tuning="auto")
        if not precond:   # the plain solve is the unpreconditioned BiCGStab
            cc.set_option("ppe_precond", 0)
            cc.set_option("ppe_solver", abi.SOLVER_BICGSTAB)
        cc.prime()
        cc.step(1)
        o = cc.download(0)
        cc.close()
        return o

    def rel(a, b):   # by particle id (cell-boundary particles may re-bin differently)
        oa, ob = np.argsort(a["pid"]), np.argsort(b["pid"])
        if not np.array_equal(a["pid"][oa], b["pid"][ob]):
            return None
        return float(np.linalg.norm(b["p"][ob] - a["p"][oa]) / np.linalg.norm(a["p"]))

    ref = one_step(abi.PREC_FP64, P[0].ppe_tol)
    res["p_rel_l2_vs_fp64"] = rel(ref, one_step(abi.PREC_MIXED, P[0].ppe_tol))
    # floor set by the solver tolerance alone: the FP64 path with the plain
    # (unpreconditioned) BiCGStab against the FP64 path, both at the same tolerance
    res["p_rel_l2_fp64_plain_vs_fp64_same_tol"] = rel(ref, one_step(abi.PREC_FP64, P[0].ppe_tol, precond=0))
    res["p_rel_l2_vs_fp64_tol1e-12"] = rel(one_step(abi.PREC_FP64, 1e-12), one_step(abi.PREC_MIXED, 1e-12))
    return res


def run_e2e(args, D, P, S, G):
    """The public API as a user runs it: the scene's arrays uploaded from
    pinned host memory into a new context, prime, then every step the step
    and a read-back of the particle state (positions, velocities, pressure,
    masses, densities, salinity, ids, flags) into pinned host arrays."""
    from beachslope_gb300 import api
    pin_in = [api.pinned_copy(s) for s in S]
    pin_out = [api.pinned_state(int(len(s["x"]) * 1.25) + 1024) for s in S]
    t0 = time.perf_counter()
    ctx = api.Context(P, pin_in, G, tuning="auto")
    ctx.prime()
    h2d = sum(len(s["x"]) * (10 * 8 + 2 * 4 + 1) for s in S)
    d2h = 0
    for _ in range(args.steps):
        ctx.step(1)
        for s in range(ctx.nscenes):
            o = ctx.download(s, full=False, out=pin_out[s])
            d2h += sum(v.nbytes for v in o.values())
    ctx.sync()
    t = time.perf_counter() - t0
    t = D.allreduce(t, "max")
    parts = D.allreduce(sum(len(s["x"]) for s in S), "sum")
    ctx.close()
    return {"value": parts * args.steps / t, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
            "d2h_bytes_per_step": int(d2h / args.steps),
            "note": "context creation, upload from pinned memory and prime inside the timed region; "
                    "state read back into pinned memory every step"}


# ------------------------------------------------------- reference arm
def run_reference(args, D, budget_s=150.0):
    """The reference's CPU path: the FP64 restatement of the reference step
    (oracle port; the Fortran reference needs MKL and gfortran, absent here),
    all host threads, on the same workload.  Steps run until K are done or
    the time budget is spent (bounded sample)."""
    from oracle import oracle
    from beachslope_gb300 import abi
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    P, S, G = build_workload(args.workload, abi.PREC_FP64)
    o = oracle.Oracle(P[0], S[0], G[0])
    o.stage("prime")
    n = o.n
    o.step(1)   # warm-up (page-in, first allocations)
    t0 = time.perf_counter()
    done = 0
    while done < args.steps and (time.perf_counter() - t0) < budget_s:
        o.step(1)
        done += 1
    t = time.perf_counter() - t0
    v = n * done / t
    return v, {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{done} production step(s) of the full {args.workload} scene ({n} particles) "
                         f"after 1 warm-up step, {t:.1f} s"}


def cpu_baseline(args):
    from oracle import oracle
    from beachslope_gb300 import abi
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    P, S, G = build_workload(args.workload, abi.PREC_FP64)
    o = oracle.Oracle(P[0], S[0], G[0])
    o.stage("prime")
    t0 = time.perf_counter()
    o.step(1)
    t = time.perf_counter() - t0
    return {"value": o.n / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"1 production step of the full {args.workload} scene ({o.n} particles), {t:.1f} s"}


def run_batched(args):
    """64 seeded beach scenes of uneven size in one context (one launch per
    stage for all of them): ISPH and WCSPH steps, mixed precision."""
    from beachslope_gb300 import abi, api, scene
    scenes = scene.batch_scenes(args.batch_scenes, precision=abi.PREC_MIXED)
    P = [s[0] for s in scenes]
    S = [s[1] for s in scenes]
    G = [s[2] for s in scenes]
    n = sum(len(s["x"]) for s in S)
    out = {"scenes": len(P), "particles": n, "particles_min": min(len(s["x"]) for s in S),
           "particles_max": max(len(s["x"]) for s in S), "steps": args.batch_steps,
           "description": "slope 1:5-1:20, A 0.02-0.10 m, porosity 0.3-0.5, dx 5-20 mm log-uniform (seeded)"}
    for mode in ("isph", "wcsph"):
        if mode == "wcsph":
            conv = [scene.to_wcsph(p, s) for p, s in zip(P, S)]
            Pm, Sm = [c[0] for c in conv], [c[1] for c in conv]
        else:
            Pm, Sm = P, S
        ctx = api.Context(Pm, Sm, G)
        ctx.prime()
        if mode == "wcsph":
            ctx.stage("wcsph_pressure_to_density")
        stepf = ctx.step if mode == "isph" else ctx.wcsph_step
        stepf(2)
        ctx.sync()
        ctx.record(0)
        stepf(args.batch_steps)
        ctx.record(1)
        ms = ctx.elapsed_ms(0, 1)
        err = [ctx.info(k)["err_bits"] for k in range(len(Pm))]
        out[mode] = {"value": n * args.batch_steps / (ms / 1e3), "unit": UNIT,
                     "ms_per_step": ms / args.batch_steps, "scenes_with_errors": int(sum(e != 0 for e in err))}
        ctx.close()
    return out


def run_serving(args):
    """Request loop: Poisson arrivals, log-uniform sizes, slot admission into
    one batched context (mixed precision); the same requests solved one at a
    time with the FP64 drop-in as the serial baseline."""
    from beachslope_gb300 import abi, api, scene, serve
    reqs = serve.poisson_requests(args.serve_requests, args.serve_rate, precision=abi.PREC_MIXED)
    steps = args.serve_steps
    classes = [(500_000, 3), (64_000, 5)]   # (largest request, slots)
    templates = []
    for cap, k in classes:
        tp, tst, tgr = scene.beach_scene(dx=scene.dx_for_particles(cap), precision=abi.PREC_MIXED)
        templates += [(tp, int(1.3 * len(tst["x"])), int(1.3 * len(tgr["x"])) + 64)] * k
    srv = serve.Server(templates)
    t0 = time.perf_counter()
    res = srv.run(reqs, steps)
    wall = time.perf_counter() - t0
    srv.close()
    lat = np.array([res[r.rid]["latency"] for r in reqs])
    psteps = sum(len(r.state["x"]) for r in reqs) * steps
    out = {"requests": len(reqs), "rate_per_s": args.serve_rate, "steps_per_request": steps,
           "particles_min": min(len(r.state["x"]) for r in reqs),
           "particles_max": max(len(r.state["x"]) for r in reqs),
           "slots": {str(c): k for c, k in classes},
           "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                         "mean": float(lat.mean())},
           "value": psteps / wall, "unit": UNIT, "wall_s": wall,
           "errors": int(sum(res[r.rid]["info"]["err_bits"] != 0 for r in reqs)),
           "note": "each request %d production steps (the configuration's 0.5 s of physical time is %d steps)"
                   % (steps, 5000)}
    # serial FP64 baseline: the same requests one after another
    t0 = time.perf_counter()
    lat_s = []
    for r in reqs:
        p = abi.Params.from_buffer_copy(r.params)
        p.precision = abi.PREC_FP64
        c = api.Context([p], [r.state], [r.grains], tuning="auto")
        c.prime()
        c.step(steps)
        c.sync()
        c.close()
        lat_s.append(time.perf_counter() - t0 - r.arrival)
    wall_s = time.perf_counter() - t0
    lat_s = np.array(lat_s)
    out["serial_fp64"] = {"value": psteps / wall_s, "unit": UNIT, "wall_s": wall_s,
                          "latency_s": {"p50": float(np.percentile(lat_s, 50)),
                                        "p99": float(np.percentile(lat_s, 99))}}
    return out


def dtype_of(precision):
    return "f64" if precision == "fp64" else "f32+f64"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="beach_dx0.00125", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison run")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-scene batched workload")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=10)
    ap.add_argument("--no-serve", action="store_true", help="skip the request-loop workload")
    ap.add_argument("--serve-requests", type=int, default=16)
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-steps", type=int, default=40)
    args = ap.parse_args()
    D = Dist()
    config = {"workload": args.workload, "description": WORKLOADS[args.workload], "dt": 1e-4,
              "ppe_tol": 1e-8, "precision": args.precision, "scenes_per_gpu": 1,
              "ppe_solver": None,
              "l2": "state larger than L2, streamed every step (no flush)"}
    base = {"metric": METRIC, "unit": UNIT, "n_gpus": D.world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic",
            "config": config}
    if args.impl == "reference":
        if D.rank == 0:
            v, cb = run_reference(args, D)
            line = dict(base)
            line.update({"impl": "reference", "value": v, "dtype": "f64", "ms_per_step": None,
                         "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                                                     "d2h_bytes_per_step": 0}})
            line["n_gpus"] = 0
            print(json.dumps(line), flush=True)
        D.close()
        return
    out = run_ours(args, D)
    if D.rank == 0:
        line = dict(base)
        line.update({"value": out["value"], "ms_per_step": out["ms_per_step"], "dtype": dtype_of(args.precision)})
        for k in ("roofline", "e2e", "gpu_launches", "clocks", "fp64"):
            if k in out:
                line[k] = out[k]
        line["config"]["particles_per_gpu"] = out["particles"]
        line["config"]["ppe_iters_last_step"] = out["ppe_iters_last"]
        line["config"]["ppe_relres_last_step"] = out["ppe_relres_last"]
        line["config"]["err_bits"] = out["err_bits"]
        line["config"]["solver_tuning"] = out["tuning"]
        tun = out["tuning"] or {}
        line["config"]["ppe_solver"] = (
            f"FGMRES({int(tun.get('ppe_restart', 150))}), multigrid right preconditioner"
            if int(tun.get("ppe_solver", 0)) == 1 else "BiCGStab, multigrid right preconditioner")
        if D.world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(args)
        if not args.no_batch:
            line["batched"] = run_batched(args)
        if not args.no_serve:
            line["serving"] = run_serving(args)
        print(json.dumps(line), flush=True)
    D.close()


if __name__ == "__main__":
    main()
