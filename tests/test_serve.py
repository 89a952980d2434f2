"""Serving path (dfg_server_*) against the CPU oracle, in the three modes:
plain FP64, FP32 factor ("fp32f") and the mixed form ("mixed": FP32 SpMV and
Krylov vectors with FP64 reliable updates).

Bars, per request:
  * status OK and true relative residual ||b - A x|| / ||b|| <= 1e-8 (the
    server's stop test);
  * solution within 1e-6 relative L2 of the oracle's FP64 solve;
  * FP64 mode: iteration count within +-2 of the oracle's unless a residual
    replacement continued the recursion (then at most 2 chunks more);
  * a request's solution is bit-identical alone and in a mix.
"""
import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu


def _stream(n, seed, nmin=300, nmax=3000):
    from delfem_gb300 import meshgen as mg
    return [it.problem() for it in mg.serve_stream_2d(nreq=n, seed=seed, nmin=nmin, nmax=nmax)]


def _serve(ctx, probs, **kw):
    from delfem_gb300.serve import Server
    with Server(ctx, **kw) as S:
        ids = [S.submit(p) for p in probs]
        res = [S.wait(i) for i in ids]
        stats = S.stats()
    return res, stats


@pytest.mark.parametrize("mode", ["fp64", "fp32f", "mixed"])
def test_serve_matches_oracle(gpu_ctx, oracle_lib, mode):
    probs = _stream(10, seed=11)
    res, stats = _serve(gpu_ctx, probs, mode=mode, chunk_iters=4)
    assert stats["finished"] == len(probs)
    for p, r in zip(probs, res):
        assert r["status"] == 0, (p.name, r)
        assert 0.0 <= r["rel_true"] <= 1e-8, (p.name, r)
        ref = oracle_lib.solve(p)
        xr = ref["x"]
        assert np.linalg.norm(r["x"] - xr) <= 1e-6 * np.linalg.norm(xr), p.name
        if mode == "fp64":
            assert ref["iter"] - 2 <= r["iterations"] <= ref["iter"] + 8, (p.name, r["iterations"], ref["iter"])


@pytest.mark.parametrize("mode", ["fp32f", "mixed"])
def test_serve_alone_equals_in_mix(gpu_ctx, mode):
    probs = _stream(8, seed=12)
    mix, _ = _serve(gpu_ctx, probs, mode=mode)
    for k in (0, 5):
        alone, _ = _serve(gpu_ctx, [probs[k]], mode=mode)
        assert alone[0]["status"] == 0
        assert np.array_equal(bits(alone[0]["x"]), bits(mix[k]["x"])), k
        assert alone[0]["iterations"] == mix[k]["iterations"]


def test_serve_budget_queues_and_rejects(gpu_ctx):
    from delfem_gb300 import capi
    from delfem_gb300 import meshgen as mg
    probs = _stream(6, seed=13, nmin=1500, nmax=3000)
    free, _ = _serve(gpu_ctx, probs, mode="fp32f")
    # room for the largest request and a little more: admission must queue
    budget = max(r["device_bytes"] for r in free) + (1 << 20)
    big = mg.rect_problem_2d(mg.SOLID2D, 60000, seed=5)
    res, stats = _serve(gpu_ctx, probs + [big], mode="fp32f", budget_bytes=budget)
    for r, f in zip(res[:-1], free):
        assert r["status"] == 0 and r["rel_true"] <= 1e-8
        assert np.array_equal(bits(r["x"]), bits(f["x"]))
    assert res[-1]["status"] == capi.DFG_OOM_REJECTED
    assert stats["peak_bytes"] <= budget
    assert stats["peak_inflight"] < len(probs)


def test_serve_size_groups_same_results(gpu_ctx):
    """Grouping solves by size changes when they iterate, not what they compute."""
    probs = _stream(8, seed=14, nmin=300, nmax=60000)
    one, _ = _serve(gpu_ctx, probs, mode="fp32f", size_groups=1)
    three, st = _serve(gpu_ctx, probs, mode="fp32f", size_groups=3)
    for a, b in zip(one, three):
        assert a["status"] == 0 and b["status"] == 0
        assert np.array_equal(bits(a["x"]), bits(b["x"])) and a["iterations"] == b["iterations"]


@pytest.mark.parametrize("mode", ["fp64", "fp32f", "mixed"])
def test_serve_sweep_kernels_agree(gpu_ctx, oracle_lib, mode):
    """The two batched sweep kernels -- ranged over several CTAs and one CTA
    per solve -- evaluate each row with the same operations in the same order,
    so a served solve gives the same bits with either; both meet the oracle
    bars (2D and 3D kinds, sizes across the stream's range)."""
    from delfem_gb300 import meshgen as mg
    probs = _stream(5, seed=15, nmin=300, nmax=40000) + [
        mg.box_problem_3d(mg.POISSON3D, 9, 8, 7, seed=4), mg.box_problem_3d(mg.SOLID3D, 6, 7, 5, seed=5)]
    ranged, _ = _serve(gpu_ctx, probs, mode=mode, sweeps=1)
    solo, _ = _serve(gpu_ctx, probs, mode=mode, sweeps=2)
    for p, a, c in zip(probs, ranged, solo):
        assert a["status"] == 0 and c["status"] == 0, (p.name, a, c)
        assert c["rel_true"] <= 1e-8
        assert np.array_equal(bits(a["x"]), bits(c["x"])) and a["iterations"] == c["iterations"], p.name
        xr = oracle_lib.solve(p)["x"]
        assert np.linalg.norm(c["x"] - xr) <= 1e-6 * np.linalg.norm(xr), p.name


def test_serve_3d_kinds(gpu_ctx, oracle_lib):
    from delfem_gb300 import meshgen as mg
    probs = [mg.box_problem_3d(mg.POISSON3D, 6, 7, 8, seed=1), mg.box_problem_3d(mg.SOLID3D, 5, 6, 7, seed=2),
             mg.rect_problem_2d(mg.SOLID2D, 900, seed=3)]
    for mode in ("fp64", "fp32f", "mixed"):
        res, _ = _serve(gpu_ctx, probs, mode=mode)
        for p, r in zip(probs, res):
            assert r["status"] == 0 and r["rel_true"] <= 1e-8, (mode, p.name, r)
            xr = oracle_lib.solve(p)["x"]
            assert np.linalg.norm(r["x"] - xr) <= 1e-6 * np.linalg.norm(xr), (mode, p.name)


def test_serve_zero_rhs_and_iteration_limit(gpu_ctx):
    from delfem_gb300 import capi
    from delfem_gb300 import meshgen as mg
    p0 = mg.rect_problem_2d(mg.POISSON2D, 500, seed=9)
    p0.params = p0.params.copy()
    p0.params[1] = 0.0
    p0.load = None
    res, _ = _serve(gpu_ctx, [p0], mode="fp64")
    assert res[0]["status"] == 0 and res[0]["iterations"] == 0 and not np.any(res[0]["x"])
    p1 = mg.rect_problem_2d(mg.SOLID2D, 2000, seed=10)
    res, _ = _serve(gpu_ctx, [p1], mode="fp64", maxit=3)
    assert res[0]["status"] == capi.DFG_NOT_CONVERGED and res[0]["iterations"] == 3
    # the mixed form: the same zero right-hand side and limit semantics
    res, _ = _serve(gpu_ctx, [p0], mode="mixed")
    assert res[0]["status"] == 0 and res[0]["iterations"] == 0 and not np.any(res[0]["x"])
    res, _ = _serve(gpu_ctx, [p1], mode="mixed", maxit=3)
    assert res[0]["status"] == capi.DFG_NOT_CONVERGED and res[0]["iterations"] == 3
