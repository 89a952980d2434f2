#!/usr/bin/env python
"""Throughput benchmark of the FE assembly + ILU(0)-PCG hot path on GB300.

Default workload (``--config serve2d``): the serving stream -- 2,000 solves,
50/50 2D Poisson (1x1 blocks) and 2D plane-strain elasticity (2x2 blocks) on
jittered triangulated rectangles, node counts log-uniform in [2k, 400k],
log-normal (sigma 0.5) per-element coefficients, 1-3 random Dirichlet sides
and one loaded side.  Every request runs AddLinSys_* -> FinalizeMarge ->
ILU(0) -> PCG to a true relative residual <= 1e-8 inside the server
(include/dfg.h, dfg_server_*), which admits requests by free device memory and
iterates all in-flight solves together in batched launches replayed from
captured CUDA graphs.  The W + K steps split the stream into equal
consecutive segments: the first W are served as warm-up, the last K as one
timed stream.  ``serve2d`` measures capacity: every timed request is
submitted at t = 0 (the stream's seeded arrival times are ignored), so the
server always has a queue (the line reports the fraction of the timed region
with requests waiting for admission).  ``serve2d_latency`` serves the same
stream at its seeded Poisson arrivals of 50 requests/s for p50/p99 latency at
a fixed load.  Arms, on the same requests: served FP32-factor mixed precision
(FP32 factor and sweeps), the FP32-SpMV mixed form (FP32 SpMV and Krylov
vectors too, FP64 reliable updates), and served plain FP64.  ``value`` is the faster of the two mixed-precision arms (named in
``serving.head_arm``); every arm's solves/s and its ratio to plain FP64 are
in the line.  Requests come from host memory and solutions return to host
memory, so ``value`` is end to end (``e2e`` repeats it with the bytes moved).  Timing is
the host clock around the timed stream with the device synchronised at both
ends (the server runs several streams and threads); per-kernel device times
come from CUDA events inside profiled graph replays.

``--config serve3d`` / ``serve3d_latency``: the 3D stream (500 solves, 3D
Poisson / elasticity on hex grids of 16-80 cells per axis, sigma 1.0,
admission budget 120 GB).  Single-solve configurations (``solid2d_1000x500``
and smaller) time one complete solve per step with three precision arms.

``--impl reference`` runs the reference's CPU algorithm (the oracle's
bit-exact restatement) on all host cores: for the serving configurations it
solves the same timed requests as the GPU arm, spread over the cores, timed
by the wall clock.
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
    # serving: `rate` is the seeded Poisson arrival rate of the stream;
    # `saturate` submits every timed request at once (capacity)
    "serve2d": dict(kind="serve", dim=2, nreq=2000, seed=4, rate=50.0, budget=0, saturate=True),
    "serve2d_latency": dict(kind="serve", dim=2, nreq=2000, seed=4, rate=50.0, budget=0, saturate=False),
    "serve3d": dict(kind="serve", dim=3, nreq=500, seed=5, rate=30.0, budget=120 * 10**9, saturate=True),
    "serve3d_latency": dict(kind="serve", dim=3, nreq=500, seed=5, rate=30.0, budget=120 * 10**9, saturate=False),
    "solid2d_1000x500": dict(kind="solid2d", nx=1000, ny=500),
    "poisson2d_128": dict(kind="poisson2d", n=128),
    "poisson2d_1000": dict(kind="poisson2d", n=1000),
    "solid3d_96": dict(kind="solid3d", n=96),
    "solid3d_48": dict(kind="solid3d", n=48),
    "solid2d_200x100": dict(kind="solid2d", nx=200, ny=100),
}
# Iterations of the full FP64 solve of a workload at an ILU fill level with
# a solver, measured with the reference's own algorithm (bit-exact CPU
# restatement, 1e-8); used to extrapolate the bounded CPU samples to whole
# solves.
REF_ITERS = {("solid2d_1000x500", 0, "pcg"): 2540, ("solid2d_1000x500", 1, "pcg"): 1389,
             ("poisson2d_128", 0, "pcg"): 132, ("solid2d_200x100", 0, "pcg"): 496,
             ("solid2d_200x100", 1, "pcg"): 270, ("solid2d_1000x500", 0, "bicgstab"): 2258,
             ("solid2d_200x100", 0, "bicgstab"): 374}


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


def max_over_ranks(v: float, world: int, device=None) -> float:
    """Max of a per-rank value over the process group (NCCL on the GPU path,
    any backend with CPU tensors); the value itself at N = 1."""
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, wall_per_rank: float, world: int, device=None) -> float:
    """Units processed by all ranks (each rank serves its own replica of the
    workload) over the slowest rank's time."""
    return units_per_rank * world / max_over_ranks(wall_per_rank, world, device)


# ------------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples during the timed region (clocks and throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        # the raw samples go to DFG_CLOCKS_DIR when set (kept for inspection),
        # else to a temporary file; the JSON line carries their summary
        d = os.environ.get("DFG_CLOCKS_DIR")
        self.temp = not d
        self.cached = None
        if d:
            self.path = os.path.join(d, f"clocks_rank{device}.csv")
        else:
            import tempfile
            fd, self.path = tempfile.mkstemp(prefix=f"dfg_clocks{device}_", suffix=".csv")
            os.close(fd)

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
        if self.cached is None:
            self.cached = self._read()
            if self.temp and os.path.exists(self.path):
                os.remove(self.path)
        return self.cached

    def _read(self):
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
    Dirichlet + ILU(k) of the full problem and `iters` PCG iterations."""
    name, iters, fill_level, solver = args
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    p = make_problem(name)
    t0 = time.perf_counter()
    out = O.solve(p, tol=1e-30, maxit=iters, fill_level=fill_level, solver=solver)
    t = time.perf_counter() - t0
    t_it = out["t_pcg"] if solver == "pcg" else out["t_solve"]
    return dict(t_assemble=out["t_assemble"], t_ilu=out["t_ilu"], t_pcg=t_it, iters=iters, wall=t)


def cpu_rate(name, iters_full, procs, sample_iters, fill_level=0, solver="pcg"):
    """Solves/s of the reference algorithm on `procs` host cores (independent
    solves, one per core), extrapolated from bounded samples."""
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    ctx = mp.get_context("spawn")
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_sample, [(name, sample_iters, fill_level, solver)] * procs)
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
    s = FESolve(ctx, p, fill_level=args.fill_level, sweep_mode=args.sweep_mode)
    sched = {1: "ranged", 2: "level-scheduled", 3: "one CTA"}
    sweeps = dict(zip(("forward", "backward"), (sched[k] for k in s.prec.GetSweepMode())))
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
        r = s.solve(mode, target_true=True, solver=args.solver)
        return ok, r

    arms_run = [(a, m) for a, m in ARMS if a in args.arms.split(",")]
    # L2 flush between timed solves: a 256 MB write (twice the 129 MB L2) on
    # the library's stream, outside each solve's CUDA events
    flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device=torch.device("cuda", local)) \
        if torch is not None else None

    def flush_l2():
        if flush_buf is not None:
            with torch.cuda.stream(ext):
                flush_buf.zero_()

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
                flush_l2()
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
        # the solves' own device time (the flushes between them excluded)
        total_ms = sum(lat) if e_all0 is not None else 1e3 * wall
        launches = ctx.kernel_launches - launches0
        results[arm] = dict(mode=mode, total_ms=total_ms, lat=lat, iters=iters, conv=convs, launches=launches,
                            clocks=clk.summary(), true_rel=s.ls.true_residual(), x=s.solution(), sweeps=sweeps)

    # per-kernel timing (CUDA events on the library's stream) + algorithmic bytes
    # of the PCG iteration's kernels (for --solver bicgstab: the sweeps and the
    # SpMV it shares with PCG, after one untimed PCG solve that sets them up)
    prof = {}
    for arm, mode in arms_run:
        s.assemble()
        s.factor()
        s.solve(mode, target_true=True)
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
        return max_over_ranks(v, world, f"cuda:{local}")

    for mode in results:
        results[mode]["total_ms"] = gmax(results[mode]["total_ms"])
    if e2e is not None:
        e2e["value"] = args.steps * world / gmax(args.steps * world / e2e["value"])

    out = None
    if rank == 0:
        out = compose_line(args, world, p, results, prof, e2e, head)
        out["config"]["sweep_schedule"] = sweeps
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


def ncu_traffic(kernel: str, algorithmic_bytes: float | None = None):
    """Per-launch DRAM bytes of `kernel` (a name, then ':' and the sweep
    schedule for sweeps, spaces as '_') from the committed ncu summary
    (profiles/ncu_traffic.txt), scaled to `algorithmic_bytes` when the
    captured launch's algorithmic bytes are recorded; None without an entry."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                dram = float(parts[1])
                cap = float(parts[2]) if len(parts) >= 3 else None
            except ValueError:
                return None
            if cap and algorithmic_bytes:
                return round(dram * algorithmic_bytes / cap)
            return round(dram)
    return None


def compose_line(args, world, p, results, prof, e2e, head):
    import numpy as np
    steps = args.steps
    hbm_peak, peak_kind = load_peaks()

    sched = (results and next(iter(results.values())).get("sweeps")) or {}

    def traffic_key(name):
        # sweeps are keyed by their schedule: the kernels differ
        if name == "sweep_fwd":
            return f"sweep_fwd:{sched.get('forward', '')}".replace(" ", "_")
        if name == "sweep_bwd":
            return f"sweep_bwd:{sched.get('backward', '')}".replace(" ", "_")
        return name

    def roof(ms, by, name):
        b = by.get(name)
        if b is None:
            return None
        achieved = b / (ms[name] * 1e-3) / 1e9
        return dict(bound="hbm", achieved=round(achieved, 1), peak=hbm_peak, unit="GB/s",
                    frac=round(achieved / hbm_peak, 4), traffic=ncu_traffic(traffic_key(name), b),
                    peak_source=peak_kind, kernel=name, ms_per_launch=round(ms[name], 4), algorithmic_bytes=int(b))

    def arm_summary(arm):
        r = results[arm]
        ms, by = prof[arm]
        return {"value": round(steps * world / (r["total_ms"] / 1e3), 4), "unit": "solves/s",
                "p50_ms": round(_pct(r["lat"], 0.5), 3), "p99_ms": round(_pct(r["lat"], 0.99), 3),
                "dof_iterations_per_s": round(sum(p.ndof * (it + 1) for it in r["iters"]) * world
                                              / (r["total_ms"] / 1e3), 1),
                "iterations": r["iters"][-1], "true_rel_residual": r["true_rel"],
                "kernels_ms": {k: round(v, 4) for k, v in ms.items()},
                "kernels_bytes": {k: int(v) for k, v in by.items()},
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
        "dtype": {"mixed_fp32_all": "f32", "plain_fp64": "f64"}.get(head, "f32 factor/sweeps, f64 SpMV/vectors"),
        "data": "synthetic (seeded jittered mesh, log-normal coefficients)",
        "config": {"workload": args.config, "nodes": p.nnode, "dof": p.ndof, "elements": p.nelem,
                   "preconditioner": f"ILU({args.fill_level})" if args.fill_level >= 0 else "ILU(no level limit)",
                   "solver": "LsSol::Solve_PCG" if args.solver == "pcg" else "LsSol::Solve_PBiCGSTAB",
                   "tol": 1e-8, "mixed_form": head,
                   "stop": ("true relative residual <= tol (all arms)" if args.solver == "pcg" else
                            "recursive relative residual <= tol (the reference's test); true one reported"),
                   "parallelism": f"replicas x{world} (independent solves per GPU)",
                   "l2": "L2 flushed (256 MB write, untimed) before every timed solve; value from the "
                         "solves' CUDA-event times"},
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
        iters_full = REF_ITERS.get((args.config, args.fill_level, args.solver)) or \
            results[("plain_fp64" if "plain_fp64" in results else head)]["iters"][-1]
        sample_iters = args.cpu_sample_iters
        rate, t_solve, res = cpu_rate(args.config, iters_full, 1, sample_iters, args.fill_level, args.solver)
        line["cpu_baseline"] = {"value": round(rate, 6), "unit": "solves/s", "cores": 1, "kind": "port",
                                "sample": f"assembly + Dirichlet + ILU({args.fill_level}) of the full workload and {sample_iters} "
                                          f"{args.solver.upper()} iterations on one host core, extrapolated to {iters_full + 1} "
                                          f"iterations ({t_solve:.1f} s per solve)"}
    return line


# ------------------------------------------------------------- serving arm

SERVE_ARMS = [("plain_fp64", "fp64"), ("mixed_fp32_factor", "fp32f"), ("mixed_fp32_all", "mixed")]


def serve_stream(name):
    from delfem_gb300 import meshgen as mg
    c = CONFIGS[name]
    if c["dim"] == 2:
        return mg.serve_stream_2d(nreq=c["nreq"], seed=c["seed"], rate=c["rate"])
    return mg.serve_stream_3d(nreq=c["nreq"], seed=c["seed"], rate=c["rate"])


def stream_segments(name, warmup, steps, serve_requests=0):
    """The stream split into warmup + steps consecutive segments: (all items,
    warm-up items, timed items) -- the same split in both arms."""
    items = serve_stream(name)
    if serve_requests:
        items = items[:serve_requests]  # a prefix of the stream (profiling runs)
    nseg = warmup + steps
    seg = [items[(len(items) * k) // nseg:(len(items) * (k + 1)) // nseg] for k in range(nseg)]
    return items, [it for sg in seg[:warmup] for it in sg], [it for sg in seg[warmup:] for it in sg]


def serve_config(args, cfg, items, timed_items, timed_probs):
    """The workload as both arms report it (identical dicts)."""
    return {"workload": args.config, "requests": len(items), "requests_timed": len(timed_items),
            "requests_per_step": round(len(timed_items) / args.steps, 1),
            "arrivals": ("all timed requests submitted at t = 0 (capacity)" if cfg["saturate"]
                         else f"seeded Poisson arrivals at {cfg['rate']:g} requests/s"),
            "kinds": "2D Poisson / plane-strain elasticity 50:50" if cfg["dim"] == 2 else "3D Poisson / elasticity 50:50",
            "tol": 1e-8, "stop": "true relative residual <= tol (every request, every arm)",
            "l2": "in-flight working set (GBs of matrices, factors, vectors) far above the 129 MB L2; no flush"}


def gen_problems(items, threads=8):
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(threads) as ex:
        return list(ex.map(lambda it: it.problem(), items))


def serve_segment(S, items, probs, saturate):
    """Submits the requests, all at once (saturate) or at their seeded
    arrival times relative to the first; returns the request ids in order."""
    ids = []
    a0 = items[0].arrival
    t0 = time.perf_counter()
    for it, p in zip(items, probs):
        if not saturate:
            dt = (it.arrival - a0) - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
        ids.append(S.submit(p))
    return ids


def run_serve(args, rank, world, local):
    import numpy as np
    from delfem_gb300 import build as B
    B.build()
    from delfem_gb300 import linsys as L
    from delfem_gb300.serve import Server
    try:
        import torch
    except Exception:
        torch = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    cfg = CONFIGS[args.config]
    items, warm_items, timed_items = stream_segments(args.config, args.warmup, args.steps, args.serve_requests)
    t_gen = time.perf_counter()
    warm_probs = gen_problems(warm_items)
    timed_probs = gen_problems(timed_items)
    t_gen = time.perf_counter() - t_gen
    ctx = L.Context(local)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        ctx.synchronize()
        if torch is not None:
            torch.cuda.synchronize(local)

    arms_run = [(a, m) for a, m in SERVE_ARMS if a in args.arms.split(",")]
    results = {}
    x_plain = {}
    for arm, mode in arms_run:
        with Server(ctx, mode=mode, budget_bytes=int(args.serve_budget) or cfg["budget"], profile_every=16,
                    max_inflight=args.max_inflight, size_groups=args.size_groups,
                    chunk_iters=args.chunk_iters) as S:
            wids = serve_segment(S, warm_items, warm_probs, cfg["saturate"])
            for i in wids:
                S.wait(i)
                S.release(i)
            st0 = S.stats()
            prof0 = S.profile()
            barrier()
            with ClockSampler(local) as clk:
                t0 = time.perf_counter()
                ids = serve_segment(S, timed_items, timed_probs, cfg["saturate"])
                S.drain()
                barrier()
                wall = time.perf_counter() - t0
            st1 = S.stats()
            res = [S.wait(i) for i in ids]
            prof1 = S.profile()
            bad = [r for r in res if r["status"] != 0]
            if bad:
                raise RuntimeError(f"{arm}: {len(bad)} requests failed, first: {bad[0]}")
            err = []
            for k, r in enumerate(res):
                if arm == "plain_fp64":
                    x_plain[k] = r["x"].copy()
                elif k in x_plain:
                    xp = x_plain[k]
                    err.append(float(np.linalg.norm(r["x"] - xp) / max(np.linalg.norm(xp), 1e-300)))
                S.release(r["id"])
            prof = {}
            for k, v in prof1.items():
                v0 = prof0.get(k, {"n": 0, "ms": 0.0, "bytes": 0.0})
                n = v["n"] - v0["n"]
                if n <= 0:
                    continue
                ms = (v["ms"] * v["n"] - v0["ms"] * v0["n"]) / n
                by = (v["bytes"] * v["n"] - v0["bytes"] * v0["n"]) / n
                prof[k] = {"n": n, "ms": ms, "bytes": by}
        lat = [r["t_done"] - r["t_submit"] for r in res]
        svc = [r["t_done"] - r["t_admit"] for r in res]
        results[arm] = dict(
            mode=mode, wall=wall, n=len(res), lat=lat, svc=svc,
            iters=[r["iterations"] for r in res], rel_true=max(r["rel_true"] for r in res),
            launches=st1["kernel_launches"] - st0["kernel_launches"], replays=st1["replays"] - st0["replays"],
            h2d=st1["h2d_bytes"] - st0["h2d_bytes"], d2h=st1["d2h_bytes"] - st0["d2h_bytes"],
            backlog_frac=(st1["backlog_seconds"] - st0["backlog_seconds"]) / wall,
            queued_frac=(st1["queued_seconds"] - st0["queued_seconds"]) / wall,
            full_frac=(st1["full_seconds"] - st0["full_seconds"]) / wall,
            inflight_avg=(st1["inflight_seconds"] - st0["inflight_seconds"]) / wall,
            symbolic_ms=1e3 * (st1["symbolic_seconds"] - st0["symbolic_seconds"]) / max(len(res), 1),
            admit_ms=1e3 * (st1["admit_seconds"] - st0["admit_seconds"]) / max(len(res), 1),
            peak_inflight=st1["peak_inflight"], peak_bytes=st1["peak_bytes"], budget=st1["budget_bytes"],
            busy=st1["busy_seconds"] - st0["busy_seconds"], prof=prof, clocks=clk.summary(),
            err_vs_plain=(max(err) if err else None),
            dof_iters=sum(p.ndof * (r["iterations"] + 1) for p, r in zip(timed_probs, res)))

    def gmax(v):
        return max_over_ranks(v, world, f"cuda:{local}")

    for arm in results:
        results[arm]["wall"] = gmax(results[arm]["wall"])
    out = None
    if rank == 0:
        out = compose_serve_line(args, world, cfg, items, timed_items, timed_probs, results, t_gen)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return out


def _cpu_serve_sample(args):
    """Reference algorithm (oracle) on whole requests of the stream, in a
    spawned process: returns the seconds each request took."""
    name, idx = args
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    items = serve_stream(name)
    out = []
    for i in idx:
        p = items[i].problem()
        t0 = time.perf_counter()
        r = O.solve(p)
        out.append((i, time.perf_counter() - t0, int(r["iter"])))
    return out


def cpu_serve_rate(name, procs, per_proc, first=0):
    """Solves/s of the reference algorithm on one host core over `per_proc`
    whole requests of the stream (requests first, first+1, ...): requests
    over summed solve seconds (the cpu_baseline leg of the GPU arm)."""
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    ctx = mp.get_context("spawn")
    jobs = [(name, [first + k * procs + j for k in range(per_proc)]) for j in range(procs)]
    t0 = time.perf_counter()
    with ctx.Pool(procs) as pool:
        res = pool.map(_cpu_serve_sample, jobs)
    wall = time.perf_counter() - t0
    times = [t for r in res for _, t, _ in r]
    return len(times) / max(sum(times), 1e-9) * procs, times, wall


def compose_serve_line(args, world, cfg, items, timed_items, timed_probs, results, t_gen):
    hbm_peak, peak_kind = load_peaks()
    steps = args.steps

    def arm_summary(arm):
        r = results[arm]
        value = r["n"] * world / r["wall"]
        return {"value": round(value, 4), "unit": "solves/s",
                "p50_ms": round(1e3 * _pct(r["lat"], 0.5), 1), "p99_ms": round(1e3 * _pct(r["lat"], 0.99), 1),
                "service_p50_ms": round(1e3 * _pct(r["svc"], 0.5), 1),
                "service_p99_ms": round(1e3 * _pct(r["svc"], 0.99), 1),
                "dof_iterations_per_s": round(r["dof_iters"] * world / r["wall"], 1),
                "iterations_median": int(_pct(r["iters"], 0.5)), "iterations_max": int(max(r["iters"])),
                "max_true_rel_residual": r["rel_true"], "gpu_launches": int(r["launches"]),
                "graph_replays": int(r["replays"]), "peak_inflight": int(r["peak_inflight"]),
                "peak_device_bytes": int(r["peak_bytes"]),
                "saturation": {"backlog_fraction": round(r["backlog_frac"], 4),
                               "admission_queue_fraction": round(r["queued_frac"], 4),
                               "device_full_fraction": round(r["full_frac"], 4),
                               "inflight_mean": round(r["inflight_avg"], 1),
                               "symbolic_ms_per_request": round(r["symbolic_ms"], 2),
                               "admission_ms_per_request": round(r["admit_ms"], 2)},
                "error_vs_fp64_rel_l2_max": r["err_vs_plain"],
                "kernels": {k: {"ms": round(v["ms"], 4), "gbs": round(v["bytes"] / (v["ms"] * 1e-3) / 1e9, 1)
                                if v["bytes"] > 0 and v["ms"] > 0 else None}
                            for k, v in sorted(r["prof"].items(), key=lambda kv: -kv[1]["ms"])}}

    arms = {arm: arm_summary(arm) for arm in results}
    # the headline is the faster served mixed-precision form; every arm and
    # its ratio to plain FP64 are in the line
    mixed_arms = [a for a in ("mixed_fp32_factor", "mixed_fp32_all") if a in results]
    head = max(mixed_arms, key=lambda a: arms[a]["value"]) if mixed_arms else next(iter(results))
    hr = results[head]
    prof = hr["prof"]
    swept = {k: v for k, v in prof.items() if v["bytes"] > 0}
    dom = max(swept, key=lambda k: swept[k]["ms"]) if swept else None
    roof = None
    if dom is not None:
        v = swept[dom]
        achieved = v["bytes"] / (v["ms"] * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(achieved / hbm_peak, 4),
                # FP32 sweeps of the 2D classes run one CTA per solve, FP64 ones ranged
                "traffic": ncu_traffic(dom + (":one_CTA" if results[head]["mode"] != "fp64" else ":ranged")
                                       if dom.startswith("sweep") else dom, v["bytes"]),
                "peak_source": peak_kind,
                "kernel": dom, "ms_per_launch": round(v["ms"], 4), "algorithmic_bytes": int(v["bytes"]),
                "launches_timed": int(v["n"])}
    value = arms[head]["value"]
    plain = arms.get("plain_fp64")
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "solves/s",
        "n_gpus": world,
        "steps": steps,
        "warmup": args.warmup,
        "ms_per_step": round(1e3 * hr["wall"] / steps, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": {"mixed_fp32_all": "f32 factor/sweeps/SpMV/Krylov vectors, f64 residual/dots/solution",
                  "plain_fp64": "f64"}.get(head, "f32 factor/sweeps, f64 SpMV/vectors/reductions"),
        "data": "synthetic (seeded request stream: jittered meshes, log-normal coefficients)",
        "config": serve_config(args, cfg, items, timed_items, timed_probs),
        "serving": {"head_arm": head, "admission_budget_bytes": int(hr["budget"]),
                    "timing": "host clock around the timed stream, device synchronised at both ends",
                    "parallelism": f"one server per GPU, x{world}", "max_inflight": args.max_inflight,
                    "chunk_iters": args.chunk_iters, "size_groups": args.size_groups, "generation_s": round(t_gen, 1),
                    "dof_timed": int(sum(p.ndof for p in timed_probs))},
        "p50_ms": arms[head]["p50_ms"],
        "p99_ms": arms[head]["p99_ms"],
        "plain_fp64": plain,
        "mixed_fp32_factor": arms.get("mixed_fp32_factor"),
        "mixed_fp32_all": arms.get("mixed_fp32_all"),
        "mixed_over_plain": round(value / plain["value"], 3) if plain else None,
        "mixed_over_plain_by_arm": {a: round(arms[a]["value"] / plain["value"], 3)
                                    for a in arms if plain and a != "plain_fp64"},
        "error_vs_fp64_rel_l2_max": hr["err_vs_plain"],
        "roofline": roof,
        "gpu_launches": int(hr["launches"]),
        "clocks": hr["clocks"],
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": int(hr["h2d"] / steps),
                "d2h_bytes_per_step": int(hr["d2h"] / steps),
                "note": "the served stream itself: requests from host memory, solutions to host memory"},
    }
    if not args.no_cpu_baseline:
        rate, times, wall = cpu_serve_rate(args.config, 1, args.cpu_serve_requests)
        line["cpu_baseline"] = {"value": round(rate, 4), "unit": "solves/s", "cores": 1, "kind": "port",
                                "sample": f"the first {len(times)} requests of the stream solved whole (assembly, "
                                          f"ILU(0), PCG to 1e-8) by the reference algorithm on one host core "
                                          f"({sum(times):.1f} s)"}
    return line


# ---------------------------------------------------------- reference arm

def run_reference(args, rank, world):
    if rank != 0:
        return None
    procs = os.cpu_count() or 1
    if CONFIGS[args.config]["kind"] == "serve":
        return run_reference_serve(args, world, procs)
    iters_full = REF_ITERS.get((args.config, args.fill_level, args.solver))
    if iters_full is None:
        iters_full = 3000
    rates = []
    t_all0 = time.perf_counter()
    for i in range(args.warmup + args.steps):
        rate, t_solve, res = cpu_rate(args.config, iters_full, procs, args.cpu_sample_iters, args.fill_level)
        if i >= args.warmup:
            rates.append(rate)
    value = statistics.median(rates)
    return {
        "metric": METRIC, "impl": "reference", "value": round(value, 6), "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered mesh, log-normal coefficients)",
        "config": {"workload": args.config, "tol": 1e-8, "preconditioner": f"ILU({args.fill_level})",
                   "parallelism": f"{procs} independent single-threaded solves (one per host core)"},
        "ms_per_step": round(1e3 * procs / value, 1),
        "cpu_baseline": {"value": round(value, 6), "unit": "solves/s", "cores": procs, "kind": "port",
                         "sample": f"per core: assembly + Dirichlet + ILU({args.fill_level}) of the full workload and "
                                   f"{args.cpu_sample_iters} {args.solver.upper()} iterations, extrapolated to {iters_full + 1} "
                                   f"iterations; the reference algorithm's bit-exact C restatement"},
        "e2e": {"value": round(value, 6), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": round(time.perf_counter() - t_all0, 1),
    }


def request_cost(it) -> float:
    """Relative one-core cost of a stream request (for balancing the cores):
    unknowns x block work x the ILU(0)-PCG iteration growth with size."""
    from delfem_gb300 import meshgen as mg
    if len(it.size) == 1:
        n = float(it.size[0])
        return n ** 1.5 * (3.5 if it.kind == mg.SOLID2D else 1.0)
    n = float(it.size[0] * it.size[1] * it.size[2])
    return n ** (4.0 / 3.0) * (9.0 if it.kind == mg.SOLID3D else 1.0)


def lpt_assign(costs, procs):
    """Longest-processing-time-first assignment of jobs to `procs` workers."""
    import heapq
    heap = [(0.0, j) for j in range(procs)]
    out = [[] for _ in range(procs)]
    for i in sorted(range(len(costs)), key=lambda i: -costs[i]):
        load, j = heapq.heappop(heap)
        out[j].append(i)
        heapq.heappush(heap, (load + costs[i], j))
    return out


def _ref_serve_worker(name, warmup, steps, serve_requests, warm_idx, idx, barrier, q):
    """One host core of the reference arm: builds its requests' problems
    (untimed), solves one small warm-up request, meets the others at the
    barrier, then solves its share of the timed requests whole."""
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    _, warm_items, timed_items = stream_segments(name, warmup, steps, serve_requests)
    probs = [(i, timed_items[i].problem()) for i in idx]
    for i in warm_idx:
        O.solve(warm_items[i].problem())
    barrier.wait()
    out = []
    for i, p in probs:
        r = O.solve(p)
        out.append((i, int(r["iter"]), bool(r["converged"]), time.perf_counter()))
    q.put(out)


def run_reference_serve(args, world, procs):
    """The reference algorithm serving the GPU arm's timed requests (the same
    stream segments) on every host core: the requests are spread over the
    cores by estimated cost (longest first), each core solves its share one
    whole request after another (assembly, Dirichlet, ILU(0), PCG to 1e-8),
    and the rate is requests over the wall clock from the moment all cores
    start until the last finishes.  Problem generation happens before the
    start."""
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    cfg = CONFIGS[args.config]
    items, warm_items, timed_items = stream_segments(args.config, args.warmup, args.steps, args.serve_requests)
    if args.ref_sample_every > 1:
        keep = list(range(0, len(timed_items), args.ref_sample_every))
    else:
        keep = list(range(len(timed_items)))
    shares = lpt_assign([request_cost(timed_items[i]) for i in keep], procs)
    shares = [[keep[k] for k in sh] for sh in shares]
    smallest = sorted(range(len(warm_items)), key=lambda i: request_cost(warm_items[i]))
    mpc = mp.get_context("spawn")
    barrier = mpc.Barrier(procs + 1)
    q = mpc.Queue()
    t_all0 = time.perf_counter()
    ws = [mpc.Process(target=_ref_serve_worker,
                      args=(args.config, args.warmup, args.steps, args.serve_requests,
                            smallest[:1], shares[j], barrier, q))
          for j in range(procs)]
    for w in ws:
        w.start()
    barrier.wait()
    t0 = time.perf_counter()
    res = [q.get() for _ in ws]
    for w in ws:
        w.join()
    done = [x for r in res for x in r]
    t_end = max((x[3] for x in done), default=t0)
    wall = max(t_end - t0, 1e-9)
    if not all(x[2] for x in done):
        raise RuntimeError("reference arm: a request did not converge")
    n = len(done)
    value = n / wall
    return {
        "metric": METRIC, "impl": "reference", "value": round(value, 4), "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded request stream: jittered meshes, log-normal coefficients)",
        "config": serve_config(args, cfg, items, timed_items, None),
        "ms_per_step": round(1e3 * wall / args.steps, 1),
        "cpu_baseline": {"value": round(value, 4), "unit": "solves/s", "cores": procs, "kind": "port",
                         "sample": (f"{n} of the {len(timed_items)} timed requests of the stream (every "
                                    f"{max(args.ref_sample_every, 1)}), solved whole by the reference algorithm's "
                                    f"bit-exact C restatement, {procs} cores (one single-threaded solver each, "
                                    f"requests balanced by estimated cost); rate = requests / wall clock "
                                    f"({wall:.1f} s)")},
        "e2e": {"value": round(value, 4), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": round(time.perf_counter() - t_all0, 1),
        "iterations_median": int(_pct([x[1] for x in done], 0.5)) if done else None,
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="serve2d", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample-iters", type=int, default=60)
    ap.add_argument("--cpu-serve-requests", type=int, default=12,
                    help="requests the one-core CPU baseline solves (serving configs)")
    ap.add_argument("--serve-requests", type=int, default=0,
                    help="serving: serve only the first N requests of the stream (0 = all; for profiling runs)")
    ap.add_argument("--serve-budget", type=float, default=0,
                    help="serving: admission budget in bytes (0 = the workload's; small for ncu replays)")
    ap.add_argument("--solver", default="pcg", choices=["pcg", "bicgstab"],
                    help="single-solve workloads: Solve_PCG or Solve_PBiCGSTAB (BiCGSTAB: arm plain_fp64 only)")
    ap.add_argument("--fill-level", type=int, default=0,
                    help="single-solve workloads: ILU fill level (CPreconditioner_ILU::SetFillInLevel; -1 = no limit)")
    ap.add_argument("--sweep-mode", type=int, default=0, choices=[0, 1, 2, 3],
                    help="single solves: triangular-sweep schedule, 0 = timed choice, 1 ranged, "
                         "2 level-scheduled, 3 one CTA")
    ap.add_argument("--max-inflight", type=int, default=256, help="serving: solves resident at once (<= 256)")
    ap.add_argument("--chunk-iters", type=int, default=8, help="serving: PCG iterations per graph replay (<= 64)")
    ap.add_argument("--size-groups", type=int, default=0, help="serving: 1 table, 2-3 size groups, 0 = server default (3)")
    ap.add_argument("--ref-sample-every", type=int, default=4,
                    help="--impl reference, serving configs: solve every n-th timed request (1 = all of them; "
                         "4, the default, keeps the run near a minute and a half on 16 cores)")
    ap.add_argument("--arms", default=",".join(sorted({a for a, _ in ARMS + SERVE_ARMS})),
                    help="comma-separated GPU arms to run (profiling runs pick one)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_env()
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif CONFIGS[args.config]["kind"] == "serve":
        line = run_serve(args, rank, world, local)
    else:
        line = run_gpu(args, rank, world, local)
    if rank == 0 and line is not None:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
