"""bench.py's JSON contract on the CPU.  The reference arm (the reference
algorithm on every host core) prints one line carrying the base contract's
keys and the `cpu_baseline` and zero-copy `e2e` objects.  The GPU arm
without a GPU exits non-zero with the CUDA error: no CPU fallback exists."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _run(*args, timeout=600):
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT, capture_output=True,
                          text=True, timeout=timeout)


def test_reference_arm_line():
    r = _run("--impl", "reference", "--config", "poisson2d_128", "--steps", "1", "--warmup", "1")
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["n_gpus"] == 1 and d["steps"] == 1
    assert d["warmup"] >= 3  # the contract's minimum, applied when fewer are asked for
    assert d["unit"] == "solves/s" and d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["workload"] == "poisson2d_128"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_serving_arm_same_requests_wall_clock():
    """The serving reference arm solves the GPU arm's timed requests (here a
    4-request prefix of the stream: one timed request) and reports the same
    workload config the GPU arm reports."""
    r = _run("--impl", "reference", "--config", "serve2d", "--serve-requests", "4", "--steps", "1", "--warmup", "3")
    assert r.returncode == 0, r.stderr[-3000:]
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 3
    import bench
    items, warm, timed = bench.stream_segments("serve2d", 3, 1, 4)
    assert len(timed) == 1 and d["config"]["requests_timed"] == 1

    class A:
        config, steps = "serve2d", 1
    ref_cfg = bench.serve_config(A, bench.CONFIGS["serve2d"], items, timed, None)
    assert d["config"] == ref_cfg
    assert "wall clock" in d["cpu_baseline"]["sample"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"]


def test_lpt_assignment_balances():
    import bench
    costs = [10.0, 9.0, 8.0, 7.0, 6.0, 5.0, 4.0, 3.0, 2.0, 1.0]
    shares = bench.lpt_assign(costs, 3)
    assert sorted(i for sh in shares for i in sh) == list(range(10))
    loads = [sum(costs[i] for i in sh) for sh in shares]
    assert max(loads) - min(loads) <= max(costs)


def test_gpu_arm_fails_loudly_without_a_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    r = _run("--config", "poisson2d_128", "--steps", "1", "--warmup", "3", timeout=300)
    assert r.returncode != 0
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert "dfg_ctx_create" in r.stderr or "CUDA" in r.stderr


def test_ncu_traffic_entries_by_schedule():
    """DRAM traffic of a kernel comes from the committed capture of the same
    kernel: sweeps are keyed by their schedule (ranged, one CTA), scaled by
    algorithmic bytes; no entry gives None rather than another kernel's."""
    import bench
    one = bench.ncu_traffic("sweep_fwd:one_CTA")
    assert one is not None and one > 0
    assert bench.ncu_traffic("sweep_fwd:one_CTA", 2 * 661524) == 2 * one
    ranged = bench.ncu_traffic("sweep_fwd:ranged")
    assert ranged is not None and ranged != one
    assert bench.ncu_traffic("sweep_bwd_b2_e4:one_CTA") is not None
    assert bench.ncu_traffic("sweep_fwd:level-scheduled") is None
    assert bench.ncu_traffic("no_such_kernel") is None
