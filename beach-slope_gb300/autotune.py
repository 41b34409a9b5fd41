"""Autotuner for the PPE solver (Krylov method, multigrid cycle shape) and
the launch shapes of the row kernels.

Measures ms/step of the real workload (CUDA events on the context's stream)
for a small staged grid -- the Krylov method (BiCGStab, or FGMRES with a
restart length), then the multigrid cycle shape (W-cycle depth,
pre-smoothing on the particle and cell levels, Jacobi damping,
coarse-correction scale, coarsest sweeps, the clustered subtree, the
second particle-level post-sweep, the exact coarse solve, the double-float
FGMRES basis, the FP64 form's cycle in FP32), the
threads per block of the neighbour sweeps and of the particle-level
multigrid kernels, then the restart length again --
and keeps the fastest configuration whose solves converged without error
bits.  The result is written to tuning.json next to this file, keyed by
precision and a particle-count bucket; Context(..., tuning="auto") applies it.

    python -m beachslope_gb300.autotune   (via __graft_entry__.load_package())
"""
import json
import math
import os

HERE = os.path.dirname(os.path.abspath(__file__))
CACHE = os.path.join(HERE, "tuning.json")
OPTIONS = ("ppe_restart", "ppe_solver", "mg_wlev", "mg_pre0", "mg_prec", "mg_post0", "mg_omega", "mg_cscale",
           "mg_coarse_sweeps", "mg_sub", "mg_exact", "fg_df", "mg_fp32", "sweep_tpb", "mg0_tpb")


def bucket(n_particles):
    """Size class of a workload: powers of 4 of the particle count."""
    return str(int(round(math.log(max(n_particles, 1), 4))))


def key(precision, n_particles, scenes=1):
    """Cache key: precision, size class and, for a batch, a scene-count class."""
    k = f"prec{precision}_n4^{bucket(n_particles)}"
    return k if scenes <= 1 else k + f"_s4^{bucket(scenes)}"


def load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def lookup(precision, n_particles, scenes=1):
    """The entry of this size class (and scene-count class); otherwise the
    single-scene entry of the nearest size class of the same precision."""
    d = load()
    for k in (key(precision, n_particles, scenes), key(precision, n_particles)):
        if k in d:
            return d[k]
    b = int(bucket(n_particles))
    near = sorted((abs(int(k.split("^")[1]) - b), k) for k in d
                  if k.startswith(f"prec{precision}_n4^") and "_s4^" not in k)
    return d[near[0][1]] if near else None


def _measure(ctx, steps):
    ctx.sync()
    ctx.record(2)
    ctx.step(steps)
    ctx.record(3)
    ms = ctx.elapsed_ms(2, 3) / steps
    info = [ctx.info(s) for s in range(ctx.nscenes)]
    ok = all(i["err_bits"] == 0 and i["ppe_iters"] > 0 for i in info)
    iters = sum(i["ppe_iters"] for i in info) / len(info)
    return ms, ok, iters


def tune(ctx, grains, steps=2, verbose=True):
    """Staged search on a primed context; returns (best options, table).

    Every candidate starts from the same snapshot of the scenes (re-uploaded
    and primed, then one untimed step that also captures the solver graph),
    so a candidate that diverges does not leave its state to the next one."""
    table = []
    snap = [ctx.download(s) for s in range(ctx.nscenes)]

    def restore():
        for s in range(ctx.nscenes):
            ctx.upload(s, snap[s], grains[s])
        ctx.clear_errors()
        ctx.prime()

    def run(opts):
        for k, v in opts.items():
            ctx.set_option(k, v)
        try:
            restore()
            ctx.step(1)
            ms, ok, iters = _measure(ctx, steps)
        except RuntimeError:
            ms, ok, iters = math.inf, False, 0
        table.append({"options": dict(opts), "ms_per_step": ms, "ok": ok, "ppe_iters": iters})
        if verbose:
            print(f"  {opts} -> {ms:.2f} ms/step, iters {iters:.0f}{'' if ok else ' (errors)'}", flush=True)
        return ms if ok else math.inf

    base = {"ppe_restart": 30, "ppe_solver": 0, "mg_wlev": 2, "mg_pre0": 1, "mg_prec": 1, "mg_omega": 0.9,
            "mg_cscale": 1.5, "mg_coarse_sweeps": 10, "mg_sub": 0, "mg_post0": 1, "fg_df": 1,
            "sweep_tpb": 256, "mg0_tpb": 256, "mg_exact": 0, "mg_fp32": 0}
    best, best_ms = dict(base), run(base)
    solver_stage = [{"ppe_solver": 0}] + [{"ppe_solver": 1, "ppe_restart": r} for r in (20, 30, 50, 80, 120)]
    stages = [
        solver_stage,
        [{"mg_wlev": w} for w in (0, 1, 2, 3, 4)],
        [{"mg_exact": 1}],
        [{"mg_pre0": a, "mg_prec": b} for a in (0, 1) for b in (0, 1)],
        [{"mg_cscale": c} for c in (1.3, 1.5, 1.7)],
        [{"mg_omega": w} for w in (0.8, 0.9, 0.95, 1.0)],
        [{"mg_coarse_sweeps": c} for c in (5, 10, 20)],
        [{"mg_sub": 1}],
        [{"mg_post0": 2}],
        [{"fg_df": 0}],
        [{"mg_fp32": 1}],   # the FP64 form's cycle in FP32 (no effect in the mixed form)
        # launch shapes: threads per block of the neighbour sweeps and of the
        # particle-level multigrid kernels (same results, different occupancy)
        [{"sweep_tpb": t} for t in (64, 128, 256)],
        [{"mg0_tpb": t} for t in (64, 128, 256)],
        solver_stage,
    ]
    for stage in stages:
        stage_best, stage_ms = best, best_ms
        for delta in stage:
            cand = dict(best)
            cand.update(delta)
            if cand == best:
                continue
            ms = run(cand)
            if ms < stage_ms:
                stage_best, stage_ms = cand, ms
        best, best_ms = stage_best, stage_ms
    for k, v in best.items():
        ctx.set_option(k, v)
    restore()
    return best, best_ms, table


def save(precision, n_particles, best, best_ms, workload, scenes=1):
    d = load()
    d[key(precision, n_particles, scenes)] = {"options": best, "ms_per_step": best_ms, "workload": workload}
    with open(CACHE, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)


def apply(ctx, precision, n_particles, scenes=1):
    t = lookup(precision, n_particles, scenes)
    if t:
        # the restart length before the method, so FGMRES storage is sized once
        for k in sorted(t["options"], key=lambda k: OPTIONS.index(k) if k in OPTIONS else len(OPTIONS)):
            ctx.set_option(k, t["options"][k])
    return t


def main():
    import argparse
    from . import abi, api, scene
    ap = argparse.ArgumentParser()
    ap.add_argument("--dx", type=float, nargs="+", default=[0.00125, 0.0025, 0.01])
    ap.add_argument("--precision", nargs="+", default=["mixed", "fp64"])
    ap.add_argument("--batch", type=int, default=0,
                    help="tune the batch of this many seeded beach scenes instead of single scenes")
    ap.add_argument("--steps", type=int, default=2, help="timed steps per candidate")
    args = ap.parse_args()
    for prec_name in args.precision:
        prec = abi.PREC_MIXED if prec_name == "mixed" else abi.PREC_FP64
        if args.batch:
            scenes = scene.batch_scenes(args.batch, precision=prec)
            P, S, G = [q[0] for q in scenes], [q[1] for q in scenes], [q[2] for q in scenes]
            ctx = api.Context(P, S, G)
            ctx.prime()
            ctx.step(2)
            n = sum(len(q["x"]) for q in S)
            print(f"{prec_name} batch of {len(P)} scenes, n={n}", flush=True)
            best, ms, _ = tune(ctx, G, steps=args.steps)
            print(f"  best {best} {ms:.2f} ms/step", flush=True)
            save(prec, n, best, ms, f"batch of {len(P)} beach scenes", scenes=len(P))
            ctx.close()
            continue
        for dx in args.dx:
            p, st, gr = scene.beach_scene(dx=dx, precision=prec)
            ctx = api.Context([p], [st], [gr])
            ctx.prime()
            ctx.step(2)
            n = len(st["x"])
            print(f"{prec_name} dx={dx} n={n}", flush=True)
            best, ms, _ = tune(ctx, [gr], steps=args.steps)
            print(f"  best {best} {ms:.2f} ms/step", flush=True)
            save(prec, n, best, ms, f"beach dx={dx}")
            ctx.close()


if __name__ == "__main__":
    main()
