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


_FP64_PEAK = None


def fp64_peak():
    """FP64 TFLOP/s of this GPU, measured once by the library's DFMA-chain probe."""
    global _FP64_PEAK
    if _FP64_PEAK is None:
        from beachslope_gb300 import api
        _FP64_PEAK = api.measure_fp64_peak()
    return _FP64_PEAK


# ------------------------------------------------------------- our arm
# Kernels bracketed by CUDA events during the timed region (the candidates for
# the dominant kernel).
TIMED_KERNELS = ("search_effpor", "bicg_it1_spmv", "bicg_it2_spmv", "mg_l0_down", "mg_l0_up",
                 "fg_arnoldi_spmv", "fg_project")
# DRAM bytes per launch measured by ncu over the algorithmic bytes of the same
# launch (ncu dram__bytes_read.sum + dram__bytes_write.sum on the 0.18 M-particle beach, mixed);
# the traffic grows with the nonzeros and rows, so the ratio scales it to the
# bench's workload.  k_it2_64 has k_it1_64's access pattern.  fg_arnoldi_spmv:
# every launch of seven solves of the double-float form (k_fg_arn1<1>) the
# mixed bench times.
TRAFFIC_RATIO = {"search_effpor": 0.46, "bicg_it1_spmv": 0.99, "bicg_it2_spmv": 0.99,
                 "mg_l0_down": 0.99, "mg_l0_up": 0.93, "fg_arnoldi_spmv": 0.90, "fg_project": 0.97}


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
            # the particle-level residual pass: values + index per nonzero;
            # input, own smoothed value, diagonal, output and count per row
            tot += nnz * (w + 4) + n * (4 * w + 4)
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
    if args.no_step_graph:
        ctx.set_option("step_graph", 0)
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
        "step_graph": bool(ctx.get_option("step_graph")),
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
            f64pk = fp64_peak()
            out["roofline"]["fp64"] = {"flops_per_launch": round(fl), "achieved_tflops": round(fl / avg_s / 1e12, 3),
                                       "peak_tflops": round(f64pk, 3),
                                       "peak_source": "measured (bs_measure_fp64_peak: dependent DFMA chains)",
                                       "frac": round(fl / avg_s / 1e12 / f64pk, 3)}
            if df:
                out["roofline"]["fp64"]["note"] = ("basis dots, projection and off-diagonal SpMV in "
                                                   "double-float on the FP32 pipe")
        out["step_roofline"] = step_roofline(ctx, kt, fg_reads, fg_launches, args, ms_timed, pk, src)
    state = ctx.download(0)
    ctx.close()
    if not args.no_e2e:
        out["e2e"] = run_e2e(args, D, P, S, G)
    if args.precision == "mixed" and not args.no_fp64:
        out["fp64"] = run_fp64_and_accuracy(args, P, S, G, state)
        out["fp64"]["trajectory_vs_fp64"] = trajectory_errors(args, P, S, G)
    return out


# Per-particle algorithmic bytes of one production step outside the PPE solve,
# stage by stage (own fields read + written once; neighbour index lists at 4 B
# per entry for each sweep that reads them): pos words are 8 B, the other
# words w (8 FP64, 4 mixed).  Stages: projection (isph.f90:17), two re-bins
# (integrator.f90:33,251), two searches (search.f90:310), two effpor
# (porous.f90:107), two eddyvis (turbulence.f90:12), int_vel
# (integrator.f90:459), assembly (isph.f90:136), comp_vel (integrator.f90:705),
# comp_pos (integrator.f90:845), freesurf (isph.f90:49), opt2_shift
# (part_shift.f90:12), densityupdate (scalar.f90:399), timestep
# (integrator.f90:885), one scalar sub-step (scalar.f90:242).
SWEEP_POS_WORDS = 6 + 12 + 4 + 4 + 2 + 2 + 2 + 6 + 4 + 2           # 44
SWEEP_W_WORDS = 3 + 32 + 16 + 14 + 18 + 16 + 12 + 13 + 3 + 1 + 10 + 6 + 2 + 11   # 157
SWEEP_LIST_READS = 2 + 2 + 1 + 1 + 1 + 1 + 1 + 1                    # index lists read (4 B per entry)


def sweep_bytes_per_particle(K, precision):
    """Algorithmic bytes per particle of one step outside the PPE solve, plus
    the assembled matrix written once ((K+1) values of 8 B and 4 B indices)."""
    w = 4 if precision == "mixed" else 8
    return SWEEP_POS_WORDS * 8 + SWEEP_W_WORDS * w + 16 + SWEEP_LIST_READS * 4 * K + K + (K + 1) * 12


def step_roofline(ctx, kt, fg_reads, fg_launches, args, ms_timed, pk, src):
    """Whole-step roofline: the algorithmic bytes of one step (the sweeps per
    particle from sweep_bytes_per_particle, plus the solver kernels' launches
    in the event-timed pass at their per-launch algorithmic bytes) over the
    measured time of a step."""
    n = sum(len(ctx.neighbour_counts(s)) for s in range(ctx.nscenes))
    K = float(np.mean(np.concatenate([ctx.neighbour_counts(s) for s in range(ctx.nscenes)])))
    sweeps = n * sweep_bytes_per_particle(K, args.precision)
    solver = 0.0
    for name in ("fg_arnoldi_spmv", "fg_project", "mg_l0_down", "mg_l0_up", "bicg_it1_spmv", "bicg_it2_spmv"):
        cnt = kt.get(name, (0, 0.0))[0]
        if cnt:
            solver += cnt * algorithmic_bytes(ctx, name, args.precision,
                                              basis_reads=fg_reads / max(fg_launches, 1))
    per_step = sweeps + solver / args.steps
    t = ms_timed / args.steps / 1e3
    return {"bound": "hbm", "achieved": round(per_step / t / 1e9, 1), "peak": pk, "peak_source": src,
            "unit": "GB/s", "frac": round(per_step / t / 1e9 / pk, 4),
            "bytes_per_step": round(per_step), "sweep_bytes_per_step": round(sweeps),
            "solver_bytes_per_step": round(solver / args.steps), "mean_neighbours": round(K, 2),
            "ms_per_step": round(ms_timed / args.steps, 3),
            "note": "time of the event-timed pass; coarse multigrid levels and scene sums counted as zero bytes"}


def trajectory_errors(args, P, S, G):
    """Mixed and FP64 from the same initial state, stepped side by side for
    the timed number of steps (each with its own tuned solver, PPE to the
    configured tolerance): rel-L2 of p, vx, vy and con between the two after
    every step, paired by particle id; max over the steps and the last."""
    from beachslope_gb300 import abi, api
    ctxs = []
    for prec in (abi.PREC_MIXED, abi.PREC_FP64):
        Q = [abi.Params.from_buffer_copy(p) for p in P]
        for q in Q:
            q.precision = prec
        c = api.Context(Q, S, G, tuning="auto")
        c.prime()
        ctxs.append(c)
    fields = ("p", "vx", "vy", "con")
    per = {f: [] for f in fields}
    for _ in range(args.steps):
        for c in ctxs:
            c.step(1)
        a, b = ctxs[0].download(0, full=False), ctxs[1].download(0, full=False)
        oa, ob = np.argsort(a["pid"]), np.argsort(b["pid"])
        if not np.array_equal(a["pid"][oa], b["pid"][ob]):
            return {"error": "particle sets differ"}
        for f in fields:
            per[f].append(float(np.linalg.norm(a[f][oa] - b[f][ob]) / max(np.linalg.norm(b[f]), 1e-300)))
    for c in ctxs:
        c.close()
    return {"steps": args.steps, "ppe_tol": P[0].ppe_tol,
            "max": {f: max(v) for f, v in per.items()}, "last": {f: v[-1] for f, v in per.items()},
            "per_step": {f: [float("%.3g" % e) for e in v] for f, v in per.items()},
            "note": "mixed vs FP64 trajectories from one initial state, compared after every step"}


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
    masses, densities, salinity, ids, flags) into pinned host arrays.  The
    read-back of step k (bs_download_async: a device snapshot, then the copy
    on a copy stream) is waited for after step k+1 is submitted, so the copy
    runs under step k+1's compute; two pinned buffers alternate."""
    from beachslope_gb300 import api
    pin_in = [api.pinned_copy(s) for s in S]
    t0 = time.perf_counter()
    ctx = api.Context(P, pin_in, G, tuning="auto")
    pin_out = [[api.pinned_state(ctx.capacity_rows(s)) for s in range(ctx.nscenes)] for _ in range(2)]
    ctx.prime()
    h2d = sum(len(s["x"]) * (10 * 8 + 2 * 4 + 1) for s in S)
    d2h = 0
    pending = []
    for k in range(args.steps):
        ctx.step(1)
        for h in pending:   # the previous step's state, copied while this step runs
            o = ctx.download_wait(h)
        pending = [ctx.download_async(s, out=pin_out[k % 2][s]) for s in range(ctx.nscenes)]
        d2h += sum(ctx.capacity_rows(s) * (10 * 8 + 2 * 4 + 1) for s in range(ctx.nscenes))
    for h in pending:
        o = ctx.download_wait(h)
    ctx.sync()
    t = time.perf_counter() - t0
    t = D.allreduce(t, "max")
    parts = D.allreduce(sum(len(s["x"]) for s in S), "sum")
    ctx.close()
    return {"value": parts * args.steps / t, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
            "d2h_bytes_per_step": int(d2h / args.steps),
            "note": "context creation, upload from pinned memory and prime inside the timed region; "
                    "state read back into pinned memory every step (bs_download_async: step k's copy "
                    "overlaps step k+1, every copy waited for inside the timed region)"}


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
    """One production step of the oracle (all host threads) on the full
    workload: the CPU baseline, and the checker of one GPU step from the same
    initial state in both precision forms (returned as a second dict)."""
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
    base = {"value": o.n / t, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"1 production step of the full {args.workload} scene ({o.n} particles), {t:.1f} s"}
    return base, oracle_parity(o, P, S, G)


def oracle_parity(o, P, S, G):
    """One production step of the GPU (FP64 drop-in and mixed form, each with
    its tuned solver) from the oracle's initial state, against the oracle's
    step: particle order and neighbour lists bit-exact (FP64), rel-L2 of p,
    vx, vy, con and the largest position difference.  Both solve the PPE to
    the workload's tolerance, so the pressure differs at the level of that
    tolerance (different Krylov methods stop at different iterates)."""
    from beachslope_gb300 import abi, api
    r = o.get()
    kmax = P[0].kmax
    co, io, do, _, _ = o.neighbours(kmax)
    out = {"steps": 1, "ppe_tol": P[0].ppe_tol, "oracle_solver": "BiCGStab (solver.f90:129-254), true-residual stop"}
    for name, prec in (("fp64", abi.PREC_FP64), ("mixed", abi.PREC_MIXED)):
        Q = abi.Params.from_buffer_copy(P[0])
        Q.precision = prec
        c = api.Context([Q], S, G, tuning="auto")
        c.prime()
        c.step(1)
        g = c.download(0)
        res = {"order_equal": bool(np.array_equal(g["pid"], r["pid"]))}
        if prec == abi.PREC_FP64:
            cg, ig, dg, _, _ = c.neighbours()
            m = np.arange(kmax)[None, :] < co[:, None]
            res["neighbour_sets_equal"] = bool(np.array_equal(cg, co) and np.array_equal(ig[m], io[m]))
            if res["neighbour_sets_equal"]:   # positions differ in the last bits after the step
                res["pair_dist_max_rel"] = float(np.max(np.abs(dg[m] - do[m]) / do[m]))
            res["mean_neighbours"] = round(float(co.mean()), 3)
            del cg, ig, dg
        og, orr = np.argsort(g["pid"]), np.argsort(r["pid"])
        if np.array_equal(g["pid"][og], r["pid"][orr]):
            for f in ("p", "vx", "vy", "con"):
                res[f"{f}_rel_l2"] = float(np.linalg.norm(g[f][og] - r[f][orr]) / max(np.linalg.norm(r[f]), 1e-300))
            res["x_max_abs"] = float(max(np.max(np.abs(g["x"][og] - r["x"][orr])),
                                         np.max(np.abs(g["y"][og] - r["y"][orr]))))
        res["ppe_iters"] = c.info(0)["ppe_iters"]
        c.close()
        out[name] = res
    out["oracle_ppe_iters"] = o.info()["ppe_iters"]
    return out


def run_config1(args):
    """The 13 k-particle beach (dx = 10 mm) over 2000 production steps: the
    FP64 drop-in and the mixed form on the GPU (CUDA events), and the oracle
    on the host cores over a bounded sample of the same steps."""
    from oracle import oracle
    from beachslope_gb300 import abi, api, scene
    steps = args.config1_steps
    out = {"workload": "beach_dx0.01", "steps": steps}
    for name, prec in (("fp64", abi.PREC_FP64), ("mixed", abi.PREC_MIXED)):
        p, st, gr = scene.beach_scene(dx=0.01, precision=prec)
        c = api.Context([p], [st], [gr], tuning="auto")
        c.prime()
        c.step(3)
        c.sync()
        c.record(0)
        c.step(steps)
        c.record(1)
        ms = c.elapsed_ms(0, 1)
        n = len(st["x"])
        out["particles"] = n
        out[name] = {"value": n * steps / (ms / 1e3), "unit": UNIT, "ms_per_step": ms / steps,
                     "err_bits": c.info(0)["err_bits"]}
        c.close()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    p, st, gr = scene.beach_scene(dx=0.01)
    o = oracle.Oracle(p, st, gr)
    o.stage("prime")
    o.step(1)
    t0 = time.perf_counter()
    done = 0
    while done < steps and time.perf_counter() - t0 < args.config1_cpu_s:
        o.step(10)
        done += 10
    t = time.perf_counter() - t0
    out["cpu_oracle"] = {"value": o.n * done / t, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{done} production steps after 1 warm-up step, {t:.1f} s"}
    return out


def run_config3(args):
    """Standalone search + PPE on the 1000 x 1000 jittered lattice (1 M
    particles, free surface on the top row, walls on three sides, N(0,1)
    source): search, effpor + int_vel, assembly and the solve to 1e-8 timed
    by CUDA events in both precision forms; neighbour sets compared, and the
    mixed pressure against the FP64 one."""
    from beachslope_gb300 import abi, api, scene
    out = {"workload": "lattice_1000x1000", "ppe_tol": 1e-8}
    sol, nb = {}, {}
    for name, prec in (("fp64", abi.PREC_FP64), ("mixed", abi.PREC_MIXED)):
        p, st, gr = scene.lattice_scene(n=1000, dx=1e-3)
        p.precision = prec
        p.ppe_tol = 1e-8
        c = api.Context([p], [st], [None], tuning="auto")
        out["particles"] = len(st["x"])
        b = np.random.default_rng(20261203).standard_normal(len(st["x"]))
        c.sync()
        c.record(0)
        c.search()
        c.record(1)
        c.porosity()
        c.int_vel()
        c.record(2)
        c.ppe_assemble()
        c.record(3)
        c.sync()
        c.set_rhs(b)
        c.record(4)
        c.ppe_solve()
        c.record(5)
        ms = [c.elapsed_ms(0, 1), c.elapsed_ms(1, 2), c.elapsed_ms(2, 3), c.elapsed_ms(4, 5)]
        inf = c.info(0)
        out[name] = {"search_ms": ms[0], "effpor_int_vel_ms": ms[1], "assemble_ms": ms[2], "solve_ms": ms[3],
                     "total_ms": sum(ms), "ppe_iters": inf["ppe_iters"], "ppe_relres": inf["ppe_relres"],
                     "err_bits": inf["err_bits"]}
        sol[name] = c.download(0, full=False)["p"]
        cnt, idx, *_ = c.neighbours()
        nb[name] = (cnt, idx)
        c.close()
    m = np.arange(nb["fp64"][1].shape[1])[None, :] < nb["fp64"][0][:, None]
    out["neighbour_sets_equal"] = bool(np.array_equal(nb["fp64"][0], nb["mixed"][0])
                                       and np.array_equal(nb["fp64"][1][m], nb["mixed"][1][m]))
    out["p_rel_l2_mixed_vs_fp64"] = float(np.linalg.norm(sol["mixed"] - sol["fp64"]) / np.linalg.norm(sol["fp64"]))
    return out


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
    final = {}
    for mode in ("isph", "isph_fp64", "wcsph"):
        if mode == "wcsph":
            conv = [scene.to_wcsph(p, s) for p, s in zip(P, S)]
            Pm, Sm = [c[0] for c in conv], [c[1] for c in conv]
        elif mode == "isph_fp64":
            Pm = [abi.Params.from_buffer_copy(p) for p in P]
            for p in Pm:
                p.precision = abi.PREC_FP64
            Sm = S
        else:
            Pm, Sm = P, S
        ctx = api.Context(Pm, Sm, G, tuning="auto")
        ctx.prime()
        if mode == "wcsph":
            ctx.stage("wcsph_pressure_to_density")
        stepf = ctx.wcsph_step if mode == "wcsph" else ctx.step
        stepf(2)
        ctx.sync()
        ctx.record(0)
        stepf(args.batch_steps)
        ctx.record(1)
        ms = ctx.elapsed_ms(0, 1)
        err = [ctx.info(k)["err_bits"] for k in range(len(Pm))]
        out[mode] = {"value": n * args.batch_steps / (ms / 1e3), "unit": UNIT,
                     "ms_per_step": ms / args.batch_steps, "scenes_with_errors": int(sum(e != 0 for e in err)),
                     "tuning": ctx.tuning["options"] if ctx.tuning else None}
        if mode != "wcsph":
            final[mode] = [ctx.download(k, full=False) for k in range(len(Pm))]
        ctx.close()
    out["isph_mixed_over_fp64"] = out["isph"]["value"] / out["isph_fp64"]["value"]
    out["isph_p_rel_l2_mixed_vs_fp64"] = batch_step_errors(P, G, final["isph"])
    return out


def batch_step_errors(P, G, states):
    """Per-step pressure error of the mixed batch against the FP64 batch: both
    restart from the same state (the mixed batch's state at the end of its
    timed steps) and take one step; per-scene rel-L2 of p by particle id, at
    the configured PPE tolerance and with both solved to 1e-12 (which
    separates the precision of the forms from the solver tolerance: two FP64
    solves by different Krylov paths differ by ~1e-6 at 1e-8)."""
    from beachslope_gb300 import abi, api
    keys = ["x", "y", "vx", "vy", "p", "mass", "rho", "oden", "ovol", "con", "tid", "pid", "flags"]
    S = [{k: st[k] for k in keys} for st in states]

    def one_step(prec, tol):
        Q = [abi.Params.from_buffer_copy(p) for p in P]
        for q in Q:
            q.precision = prec
            if tol is not None:
                q.ppe_tol = tol
                q.ppe_maxit = 20000
        c = api.Context(Q, S, G, tuning="auto")
        c.prime()
        c.step(1)
        out = [c.download(k, full=False) for k in range(len(Q))]
        c.close()
        return out

    def errors(ga, gb):
        errs = []
        for a, b in zip(ga, gb):
            oa, ob = np.argsort(a["pid"]), np.argsort(b["pid"])
            if np.array_equal(a["pid"][oa], b["pid"][ob]):
                errs.append(float(np.linalg.norm(a["p"][oa] - b["p"][ob]) / max(np.linalg.norm(b["p"]), 1e-300)))
        return errs

    errs = errors(one_step(abi.PREC_MIXED, None), one_step(abi.PREC_FP64, None))
    tight = errors(one_step(abi.PREC_MIXED, 1e-12), one_step(abi.PREC_FP64, 1e-12))
    return {"scenes_compared": len(errs), "max": max(errs) if errs else None,
            "median": float(np.median(errs)) if errs else None,
            "max_tol1e-12": max(tight) if tight else None,
            "median_tol1e-12": float(np.median(tight)) if tight else None,
            "note": "one step of both forms from the mixed batch's state after its timed steps, at the "
                    "configured tolerance and with both solved to 1e-12"}


def run_serving(args):
    """Request loop: Poisson arrivals, log-uniform sizes, slot admission into
    one batched context (mixed precision); the same requests solved one at a
    time with the FP64 drop-in as the serial baseline."""
    from beachslope_gb300 import abi, api, scene, serve
    reqs = serve.poisson_requests(args.serve_requests, args.serve_rate, precision=abi.PREC_MIXED)
    steps = args.serve_steps
    # size classes (largest request of the class, share of the memory budget,
    # concurrency limit): the slot table is laid out within half of the free
    # device memory at the device bytes per row measured on a calibration context
    spec = [(500_000, 0.85, args.serve_large_slots), (64_000, 0.15, args.serve_small_slots)]
    classes = []
    for cap, share, limit in spec:
        tp, tst, tgr = scene.beach_scene(dx=scene.dx_for_particles(cap), precision=abi.PREC_MIXED)
        classes.append((tp, int(1.3 * len(tst["x"])), int(1.3 * len(tgr["x"])) + 64, share, limit))
        if cap == spec[0][0]:
            bpr = serve.Server.calibrate(tp, tst, tgr, tuning="auto")
    free0, total = api.device_memory()
    srv = serve.Server.for_memory(classes, bpr, budget_bytes=0.5 * free0, tuning="auto")
    t0 = time.perf_counter()
    res = srv.run(reqs, steps)
    wall = time.perf_counter() - t0
    held = srv.ctx.device_bytes()
    srv.close()
    done = [r for r in reqs if "latency" in res[r.rid]]
    lat = np.array([res[r.rid]["latency"] for r in done])
    psteps = sum(len(r.state["x"]) for r in done) * steps
    out = {"requests": len(reqs), "rate_per_s": args.serve_rate, "steps_per_request": steps,
           "particles_min": min(len(r.state["x"]) for r in reqs),
           "particles_max": max(len(r.state["x"]) for r in reqs),
           "slots": {str(c[0]): k for c, k in zip(spec, srv.class_counts)},
           "memory": {"device_free_bytes": int(free0), "device_total_bytes": int(total),
                      "budget_bytes": int(srv.budget_bytes), "planned_bytes": int(srv.planned_bytes),
                      "context_bytes": int(held), "bytes_per_row": round(bpr, 1),
                      "limits": {str(c[0]): c[2] for c in spec},
                      "binding": {str(c[0]): ("memory" if k < c[2] else "concurrency limit")
                                  for c, k in zip(spec, srv.class_counts)}},
           "rejected": len(srv.rejected),
           "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                         "mean": float(lat.mean())},
           "value": psteps / wall, "unit": UNIT, "wall_s": wall,
           "offered_particle_steps_per_s": args.serve_rate * float(np.mean([len(r.state["x"]) for r in reqs])) * steps,
           "load": args.serve_rate * float(np.mean([len(r.state["x"]) for r in reqs])) * steps / (psteps / wall),
           "errors": int(sum(res[r.rid]["info"]["err_bits"] != 0 for r in done)),
           "error_bits": sorted({int(res[r.rid]["info"]["err_bits"]) for r in done} - {0}),
           "error_requests": [{"n": len(r.state["x"]), "bits": int(res[r.rid]["info"]["err_bits"]),
                               "iters": int(res[r.rid]["info"]["ppe_iters"])}
                              for r in done if res[r.rid]["info"]["err_bits"]][:8],
           "note": "each request %d production steps (the configuration's 0.5 s of physical time is %d steps, "
                   "an offered load of ~%.0fx what one GB300 steps, with no steady state); load = offered "
                   "particle-steps/s over the measured throughput" % (steps, 5000, 5000 / steps * args.serve_rate
                   * float(np.mean([len(r.state["x"]) for r in reqs])) * steps / (psteps / wall))}
    # serial FP64 baseline: the same requests one after another
    t0 = time.perf_counter()
    lat_s = []
    for r in done:
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
    ap.add_argument("--no-step-graph", action="store_true",
                    help="launch the stages one by one instead of one captured graph per step")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-scene batched workload")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=200)
    ap.add_argument("--no-serve", action="store_true", help="skip the request-loop workload")
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-large-slots", type=int, default=6)
    ap.add_argument("--serve-small-slots", type=int, default=12)
    ap.add_argument("--no-config1", action="store_true", help="skip the 13 k-particle 2000-step leg")
    ap.add_argument("--config1-steps", type=int, default=2000)
    ap.add_argument("--config1-cpu-s", type=float, default=10.0)
    ap.add_argument("--no-config3", action="store_true", help="skip the standalone 1 M search + PPE leg")
    ap.add_argument("--no-oracle-parity", action="store_true")
    ap.add_argument("--serve-rate", type=float, default=20.0)
    ap.add_argument("--serve-steps", type=int, default=10)
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
        for k in ("roofline", "step_roofline", "e2e", "gpu_launches", "step_graph", "clocks", "fp64"):
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
            line["cpu_baseline"], par = cpu_baseline(args)
            if not args.no_oracle_parity:
                line["oracle_parity"] = par
        if not args.no_config1:
            line["config1"] = run_config1(args)
        if not args.no_config3:
            line["config3"] = run_config3(args)
        if not args.no_batch:
            line["batched"] = run_batched(args)
        if not args.no_serve:
            line["serving"] = run_serving(args)
        print(json.dumps(line), flush=True)
    D.close()


if __name__ == "__main__":
    main()
