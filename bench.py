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
SPMV_KERNELS = {"bicg_it1_spmv": 17, "bicg_it2_spmv": 18, "mx_it1_spmv": 26, "mx_it2_spmv": 27}


def spmv_algorithmic_bytes(ctx, P, kernel):
    """Compulsory bytes of one SpMV-type BiCGStab launch over all scenes:
    per row its neighbour entries (column index 4 B + value w_A), diagonal,
    count, and the row's own vector reads/writes; neighbour vector gathers
    are counted as on-chip hits."""
    tot = 0.0
    for s in range(ctx.nscenes):
        c = ctx.neighbour_counts(s)
        nnz = float(c.sum())
        n = float(len(c))
        if kernel.startswith("bicg"):
            wa, wv = 8, 8
            vec = (3 * wv + 2 * wv + wv) if "it1" in kernel else (2 * wv + 2 * wv)
        else:
            wa, wv = 4, 4
            vec = (3 * wv + 2 * wv + wv) if "it1" in kernel else (2 * wv + 2 * wv)
        tot += nnz * (4 + wa) + n * (8 + 4 + vec)
    return tot


def run_ours(args, D):
    from beachslope_gb300 import abi, api
    api.set_device(D.local)
    prec = abi.PREC_MIXED if args.precision == "mixed" else abi.PREC_FP64
    P, S, G = build_workload(args.workload, prec)
    n_particles = sum(len(s["x"]) for s in S)
    ctx = api.Context(P, S, G)
    ctx.prime()
    for _ in range(args.warmup):
        ctx.step(1)
    ctx.sync()
    # per-kernel events only on the SpMV kernels (the dominant ones)
    mask = sum(1 << k for k in SPMV_KERNELS.values())
    ctx.kernel_timing(mask)
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
    kt = ctx.kernel_times()
    ctx.kernel_timing(0)
    ms_max = D.allreduce(ms, "max")
    parts = D.allreduce(n_particles, "sum")
    info = [ctx.info(s) for s in range(ctx.nscenes)]
    iters = float(np.mean([i["ppe_iters"] for i in info]))
    out = {
        "value": parts * args.steps / (ms_max / 1e3),
        "ms_per_step": ms_max / args.steps,
        "particles": n_particles,
        "gpu_launches": int(l1 - l0),
        "clocks": ck,
        "ppe_iters_last": iters,
        "ppe_relres_last": max(i["ppe_relres"] for i in info),
        "err_bits": int(np.bitwise_or.reduce([i["err_bits"] for i in info])),
    }
    # roofline of the dominant kernel (SpMV of the Krylov loop)
    best = None
    for name, (cnt, tms) in kt.items():
        if name in SPMV_KERNELS and cnt:
            if best is None or tms > best[2]:
                best = (name, cnt, tms)
    if best:
        name, cnt, tms = best
        alg = spmv_algorithmic_bytes(ctx, P, name)
        avg_s = tms / cnt / 1e3
        pk, src = peaks()
        achieved = alg / avg_s / 1e9
        out["roofline"] = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": pk,
                           "peak_source": src, "unit": "GB/s", "frac": round(achieved / pk, 4),
                           "traffic": None, "algorithmic_bytes_per_launch": alg,
                           "avg_launch_us": round(avg_s * 1e6, 2), "launches": cnt,
                           "share_of_step": round(sum(v[1] for k, v in kt.items() if k in SPMV_KERNELS)
                                                  / ms, 3)}
    ctx.close()
    # e2e through the C-ABI with host buffers: upload + prime inside the timed
    # region, every step followed by a device->host read of the output fields
    if not args.no_e2e:
        out["e2e"] = run_e2e(args, D, P, S, G)
    return out


def run_e2e(args, D, P, S, G):
    from beachslope_gb300 import api
    t0 = time.perf_counter()
    ctx = api.Context(P, S, G)
    ctx.prime()
    h2d = sum(len(s["x"]) * (10 * 8 + 2 * 4 + 1) for s in S)
    d2h = 0
    for _ in range(args.steps):
        ctx.step(1)
        for s in range(ctx.nscenes):
            o = ctx.download(s, full=False)
            d2h += sum(v.nbytes for v in o.values())
    ctx.sync()
    t = time.perf_counter() - t0
    t = D.allreduce(t, "max")
    parts = D.allreduce(sum(len(s["x"]) for s in S), "sum")
    ctx.close()
    return {"value": parts * args.steps / t, "unit": UNIT, "h2d_bytes_per_step": int(h2d / args.steps),
            "d2h_bytes_per_step": int(d2h / args.steps),
            "note": "upload + warm-up inside the timed region; state read back every step"}


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


def dtype_of(precision):
    return "f64" if precision == "fp64" else "f32+f64"


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="beach_dx0.00125", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    D = Dist()
    config = {"workload": args.workload, "description": WORKLOADS[args.workload], "dt": 1e-4,
              "ppe_tol": 1e-8, "precision": args.precision, "scenes_per_gpu": 1,
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
        for k in ("roofline", "e2e", "gpu_launches", "clocks"):
            if k in out:
                line[k] = out[k]
        line["config"]["particles_per_gpu"] = out["particles"]
        line["config"]["ppe_iters_last_step"] = out["ppe_iters_last"]
        line["config"]["ppe_relres_last_step"] = out["ppe_relres_last"]
        line["config"]["err_bits"] = out["err_bits"]
        if D.world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(args)
        print(json.dumps(line), flush=True)
    D.close()


if __name__ == "__main__":
    main()
