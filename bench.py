#!/usr/bin/env python
"""Throughput benchmark of the FE assembly + ILU(0)-PCG hot path on GB300.

Workload (one "step" = one complete solve): the 2D plane-strain elasticity
configuration -- 1000 x 500 cells, jittered P1 triangles (501,501 nodes,
1,003,002 DOF, 2x2 block-CRS in FP64), E = 1 with a seeded log-normal
(sigma 0.5) per-element multiplier, nu = 0.3, left edge clamped, downward
traction 1e-3 on the right edge.  A step runs InitializeMarge ->
AddLinSys_LinearSolid2D_Static -> FinalizeMarge (resident load + Dirichlet)
-> ILU(0) numeric factorisation -> PCG to a 1e-8 relative residual.

Three GPU arms solve the same inputs to the same stopping rule (true relative
residual ||b - A x|| / ||b|| <= 1e-8):
  * plain FP64 ILU(0)-PCG (``plain_fp64``);
  * mixed, FP32 factor: FP32 ILU factor and triangular sweeps, FP64 SpMV,
    vectors and reductions (``mixed_fp32_factor``);
  * mixed, all FP32: FP32 factor, sweeps, SpMV and Krylov vectors inside FP64
    refinement with FP64 reductions and solution (``mixed_fp32_all``).
``value`` is the faster of the two mixed forms (named in config.mixed_form).  Inputs (mesh,
coefficients, loads) are resident in HBM for ``value``; ``e2e`` repeats the
step through the C ABI with the per-solve inputs (element coefficients and
nodal loads) copied in from pinned host memory and the solution copied back.
The matrix (112 MB), factor records and vectors exceed the 129 MB L2, so no
separate L2 flush is needed.

``--impl reference`` times the reference's CPU algorithm (the oracle's
bit-exact restatement) on all host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PCG solves/s at 1e-8 rel. residual, served mixed vs plain FP64 GPU; p50/p99 ms"
CONFIGS = {
    # name -> (meshgen factory kwargs, description)
    "solid2d_1000x500": dict(kind="solid2d", nx=1000, ny=500),
    "poisson2d_128": dict(kind="poisson2d", n=128),
    "solid3d_96": dict(kind="solid3d", n=96),
    "solid3d_48": dict(kind="solid3d", n=48),
    "solid2d_200x100": dict(kind="solid2d", nx=200, ny=100),
}
# PCG iterations of the full FP64 solve of the default workload, measured with
# the reference's own algorithm (bit-exact CPU restatement, 1e-8); used to
# extrapolate the bounded CPU samples to whole solves.
REF_ITERS = {"solid2d_1000x500": 2540, "poisson2d_128": 132, "solid2d_200x100": None}


# (name in the JSON line, solver mode)
ARMS = [("plain_fp64", "fp64"), ("mixed_fp32_factor", "fp32f"), ("mixed_fp32_all", "mixed")]


def make_problem(name):
    from delfem_gb300 import meshgen as mg
    c = CONFIGS[name]
    if c["kind"] == "solid2d":
        return mg.solid2d_cantilever(c["nx"], c["ny"])
    if c["kind"] == "poisson2d":
        return mg.poisson2d_square(c["n"])
    if c["kind"] == "solid3d":
        return mg.solid3d_cube(c["n"])
    raise ValueError(name)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_rank{device}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- CPU baseline

def _cpu_sample(args):
    """Bounded CPU sample of one solve (runs in a spawned process): assembly +
    Dirichlet + ILU(0) of the full problem and `iters` PCG iterations."""
    name, iters = args
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    p = make_problem(name)
    t0 = time.perf_counter()
    out = O.solve(p, tol=1e-30, maxit=iters)
    t = time.perf_counter() - t0
    return dict(t_assemble=out["t_assemble"], t_ilu=out["t_ilu"], t_pcg=out["t_pcg"], iters=iters, wall=t)


def cpu_rate(name, iters_full, procs, sample_iters):
    """Solves/s of the reference algorithm on `procs` host cores (independent
    solves, one per core), extrapolated from bounded samples."""
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_sample, [(name, sample_iters)] * procs)
    per = []
    for r in res:
        t_it = r["t_pcg"] / max(r["iters"], 1)
        per.append(r["t_assemble"] + r["t_ilu"] + t_it * (iters_full + 1))
    t_solve = statistics.median(per)
    return procs / t_solve, t_solve, res


# ------------------------------------------------------------------- GPU arm

def run_gpu(args, rank, world, local):
    import numpy as np
    from delfem_gb300 import build as B
    B.build()
    from delfem_gb300 import linsys as L
    from delfem_gb300.solver import FESolve

    torch = None
    if world > 1:
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    try:
        import torch  # noqa: F811
    except Exception:
        torch = None

    p = make_problem(args.config)
    ctx = L.Context(local)
    s = FESolve(ctx, p)
    stream = ctx.stream

    def ev():
        return torch.cuda.Event(enable_timing=True) if torch is not None else None

    ext = torch.cuda.ExternalStream(stream, device=torch.device("cuda", local)) if torch is not None else None

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        ctx.synchronize()
        if torch is not None:
            torch.cuda.synchronize(local)

    def step(mode):
        s.assemble()
        ok = s.factor()
        r = s.solve(mode, target_true=True)
        return ok, r

    arms_run = [(a, m) for a, m in ARMS if a in args.arms.split(",")]
    results = {}
    for arm, mode in arms_run:
        for _ in range(args.warmup):
            step(mode)
        barrier()
        lat = []
        iters, convs = [], []
        launches0 = ctx.kernel_launches
        e_all0, e_all1 = ev(), ev()
        with ClockSampler(local) as clk:
            if e_all0 is not None:
                e_all0.record(ext)
            t0 = time.perf_counter()
            for _ in range(args.steps):
                e0, e1 = ev(), ev()
                if e0 is not None:
                    e0.record(ext)
                ok, r = step(mode)
                if e1 is not None:
                    e1.record(ext)
                    e1.synchronize()
                    lat.append(e0.elapsed_time(e1))
                else:
                    lat.append(1e3 * (time.perf_counter() - t0) - sum(lat))
                iters.append(r["iter"])
                convs.append(r["conv"])
                if not r["converged"]:
                    raise RuntimeError(f"{arm} solve did not converge: {r}")
            if e_all1 is not None:
                e_all1.record(ext)
            barrier()
            wall = time.perf_counter() - t0
        total_ms = e_all0.elapsed_time(e_all1) if e_all0 is not None else 1e3 * wall
        launches = ctx.kernel_launches - launches0
        results[arm] = dict(mode=mode, total_ms=total_ms, lat=lat, iters=iters, conv=convs, launches=launches,
                            clocks=clk.summary(), true_rel=s.ls.true_residual(), x=s.solution())

    # per-kernel timing (CUDA events on the library's stream) + algorithmic bytes
    prof = {}
    for arm, mode in arms_run:
        step(mode)
        ms, by = L.profile_kernels(s.ls, s.prec, mode, reps=10)
        prof[arm] = (ms, by)
    mixed_run = [a for a in ("mixed_fp32_factor", "mixed_fp32_all") if a in results] or list(results)
    head = max(mixed_run, key=lambda a: -results[a]["total_ms"])

    # end to end through the C ABI: per-solve inputs from pinned host memory
    e2e = None
    if True:  # every rank measures its own e2e replica
        if torch is not None:
            coef_h = torch.empty(p.nelem, dtype=torch.float64, pin_memory=True).numpy()
            load_h = torch.empty(p.ndof, dtype=torch.float64, pin_memory=True).numpy()
            x_h = torch.empty(p.ndof, dtype=torch.float64, pin_memory=True).numpy()
        else:
            coef_h, load_h, x_h = np.empty(p.nelem), np.empty(p.ndof), np.empty(p.ndof)
        coef_h[:] = p.coef if p.coef is not None else 1.0
        load_h[:] = p.load if p.load is not None else 0.0
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            s.ls.set_coef(coef_h)
            s.ls.SetLoad(load_h)
            ok, r = step(results[head]["mode"])
            x_h[:] = s.solution()
        barrier()
        e2e_wall = time.perf_counter() - t0
        e2e = dict(value=args.steps * world / e2e_wall, h2d=(coef_h.nbytes + load_h.nbytes), d2h=x_h.nbytes)

    # max over ranks
    def gmax(v):
        if world > 1:
            t = torch.tensor([v], dtype=torch.float64, device=f"cuda:{local}")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            return float(t.item())
        return v

    for mode in results:
        results[mode]["total_ms"] = gmax(results[mode]["total_ms"])
    if e2e is not None:
        e2e["value"] = args.steps * world / gmax(args.steps * world / e2e["value"])

    out = None
    if rank == 0:
        out = compose_line(args, world, p, results, prof, e2e, head)
    s.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return out


def _pct(v, q):
    v = sorted(v)
    k = max(0, min(len(v) - 1, int(round(q * (len(v) - 1)))))
    return v[k]


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


def compose_line(args, world, p, results, prof, e2e, head):
    import numpy as np
    steps = args.steps
    hbm_peak, peak_kind = load_peaks()

    def roof(ms, by, name):
        b = by.get(name)
        if b is None:
            return None
        achieved = b / (ms[name] * 1e-3) / 1e9
        return dict(bound="hbm", achieved=round(achieved, 1), peak=hbm_peak, unit="GB/s",
                    frac=round(achieved / hbm_peak, 4), traffic=ncu_traffic(name), peak_source=peak_kind,
                    kernel=name, ms_per_launch=round(ms[name], 4), algorithmic_bytes=int(b))

    def arm_summary(arm):
        r = results[arm]
        ms, by = prof[arm]
        return {"value": round(steps * world / (r["total_ms"] / 1e3), 4), "unit": "solves/s",
                "p50_ms": round(_pct(r["lat"], 0.5), 3), "p99_ms": round(_pct(r["lat"], 0.99), 3),
                "iterations": r["iters"][-1], "true_rel_residual": r["true_rel"],
                "kernels_ms": {k: round(v, 4) for k, v in ms.items()},
                "spmv_roofline": roof(ms, by, "spmv"), "gpu_launches": int(r["launches"])}

    arms = {arm: arm_summary(arm) for arm in results}
    hr = results[head]
    ms_h, by_h = prof[head]
    dom = max(ms_h, key=ms_h.get)  # every kernel launches once per iteration
    roof_dom = roof(ms_h, by_h, dom) if dom in by_h else roof(ms_h, by_h, "spmv")
    value = arms[head]["value"]
    plain = arms.get("plain_fp64", arms[head])
    xp = results["plain_fp64"]["x"] if "plain_fp64" in results else results[head]["x"]
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": world,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": round(hr["total_ms"] / steps, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32" if head == "mixed_fp32_all" else "f32 factor/sweeps, f64 SpMV/vectors",
        "data": "synthetic (seeded jittered mesh, log-normal coefficients)",
        "config": {"workload": args.config, "nodes": p.nnode, "dof": p.ndof, "elements": p.nelem,
                   "tol": 1e-8, "stop": "true relative residual <= tol (all arms)", "mixed_form": head,
                   "parallelism": f"replicas x{world} (independent solves per GPU)",
                   "l2": "working set (matrix 112 MB + factor records + vectors) larger than the 129 MB L2; no flush"},
        "p50_ms": arms[head]["p50_ms"],
        "p99_ms": arms[head]["p99_ms"],
        "iterations": arms[head]["iterations"],
        "true_rel_residual": hr["true_rel"],
        "plain_fp64": arms.get("plain_fp64"),
        "mixed_fp32_factor": arms.get("mixed_fp32_factor"),
        "mixed_fp32_all": arms.get("mixed_fp32_all"),
        "mixed_over_plain": round(value / plain["value"], 3),
        "roofline": roof_dom,
        "gpu_launches": int(hr["launches"]),
        "clocks": hr["clocks"],
        "error_vs_fp64_rel_l2": {arm: float(np.linalg.norm(results[arm]["x"] - xp) / max(np.linalg.norm(xp), 1e-300))
                                 for arm in results},
    }
    if e2e is not None:
        line["e2e"] = {"value": round(e2e["value"], 4), "unit": "solves/s", "h2d_bytes_per_step": int(e2e["h2d"]),
                       "d2h_bytes_per_step": int(e2e["d2h"])}
    if not args.no_cpu_baseline:
        iters_full = REF_ITERS.get(args.config) or results[("plain_fp64" if "plain_fp64" in results else head)]["iters"][-1]
        sample_iters = args.cpu_sample_iters
        rate, t_solve, res = cpu_rate(args.config, iters_full, 1, sample_iters)
        line["cpu_baseline"] = {"value": round(rate, 6), "unit": "solves/s", "cores": 1, "kind": "port",
                                "sample": f"assembly + Dirichlet + ILU(0) of the full workload and {sample_iters} "
                                          f"PCG iterations on one host core, extrapolated to {iters_full + 1} "
                                          f"iterations ({t_solve:.1f} s per solve)"}
    return line


# ---------------------------------------------------------- reference arm

def run_reference(args, rank, world):
    if rank != 0:
        return None
    procs = os.cpu_count() or 1
    iters_full = REF_ITERS.get(args.config)
    if iters_full is None:
        iters_full = 3000
    rates = []
    t_all0 = time.perf_counter()
    for i in range(args.warmup + args.steps):
        rate, t_solve, res = cpu_rate(args.config, iters_full, procs, args.cpu_sample_iters)
        if i >= args.warmup:
            rates.append(rate)
    value = statistics.median(rates)
    return {
        "metric": METRIC, "impl": "reference", "value": round(value, 6), "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered mesh, log-normal coefficients)",
        "config": {"workload": args.config, "tol": 1e-8,
                   "parallelism": f"{procs} independent single-threaded solves (one per host core)"},
        "ms_per_step": round(1e3 * procs / value, 1),
        "cpu_baseline": {"value": round(value, 6), "unit": "solves/s", "cores": procs, "kind": "port",
                         "sample": f"per core: assembly + Dirichlet + ILU(0) of the full workload and "
                                   f"{args.cpu_sample_iters} PCG iterations, extrapolated to {iters_full + 1} "
                                   f"iterations; the reference algorithm's bit-exact C restatement"},
        "e2e": {"value": round(value, 6), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": round(time.perf_counter() - t_all0, 1),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="solid2d_1000x500", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-iters", type=int, default=60)
    ap.add_argument("--arms", default=",".join(a for a, _ in ARMS),
                    help="comma-separated GPU arms to run (profiling runs pick one)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        line = run_gpu(args, rank, world, local)
    if rank == 0 and line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
