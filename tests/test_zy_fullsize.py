"""Parity at the sizes the performance numbers are quoted on, against the CPU
oracle (the reference algorithm's bit-exact C restatement) run on the same
generated inputs:

  * the 1000 x 500 plane-strain cantilever (501,501 nodes, 2x2 blocks,
    log-normal sigma 0.5 moduli, clamped left edge, traction on the right);
  * the 96^3 Kuhn-tetrahedra cube (912,673 nodes, 3x3 blocks, sigma 1.0,
    clamped bottom face, body force);
  * two >= 300k-node requests of the 2D serving stream (a Poisson and an
    elasticity one), served alone by the server.

Bars (solver_ls_iter.cpp:100-172 is the reference solve):
  * pattern, assembled matrix, finalized right-hand side and ILU(0) factor
    bit-identical (compared as SHA-256 digests of the arrays);
  * FP64 Solve_PCG: iterations within +-2 of the oracle's and solution within
    1e-6 relative L2 of the oracle's solution;
  * FP32-factor and FP32-SpMV mixed solves: true relative residual
    ||b - A x|| / ||b|| <= 1e-8 and solution within 1e-6 relative L2 of the
    oracle's;
  * served requests: status OK, true relative residual <= 1e-8, solution
    within 1e-6 of the oracle's, FP64-mode iterations within [-2, +8] of the
    oracle's (the server checks the true residual after a converged chunk).

The oracle solves run in spawned worker processes while the GPU works (about
two and a half minutes for the 96^3 cube on one core); the file sorts late so
that a failure here leaves the rest of the suite already run under -x.
"""
import concurrent.futures as cf
import hashlib
import multiprocessing as mp

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STREAM = dict(nreq=2000, seed=4, rate=50.0)
SPECS = {
    "solid2d_1000x500": ("solid2d_cantilever", dict(nx=1000, ny=500)),
    "solid3d_96": ("solid3d_cube", dict(n=96)),
    "serve2d_req12_poisson_376k": ("stream2d", dict(STREAM, index=12)),
    "serve2d_req48_solid_351k": ("stream2d", dict(STREAM, index=48)),
}


def _h(a, dtype):
    return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()


def _rel(x, xr):
    return float(np.linalg.norm(x - xr) / np.linalg.norm(xr))


@pytest.fixture(scope="module")
def oracle_runs():
    import oracle
    oracle.build()
    ex = cf.ProcessPoolExecutor(len(SPECS), mp_context=mp.get_context("spawn"))
    futs = {k: ex.submit(oracle.solve_digest, spec) for k, spec in SPECS.items()}
    yield futs
    ex.shutdown(wait=True, cancel_futures=True)


def _ref(oracle_runs, name):
    r = oracle_runs[name].result(timeout=3600)
    assert r["converged"] and r["ilu_rc"] == 0
    return r


@pytest.mark.parametrize("name", ["solid2d_1000x500", "solid3d_96"])
def test_fullsize_single_solve(gpu_ctx, oracle_runs, name):
    import oracle
    from delfem_gb300.solver import FESolve
    p = oracle.make_problem(SPECS[name])
    s = FESolve(gpu_ctx, p)
    rowptr, colind = s.ls.pattern()
    s.assemble()
    diag, offd = s.ls.GetMatrix()
    got = dict(rowptr=_h(rowptr, np.int32), colind=_h(colind, np.int32), diag=_h(diag, np.float64),
               offd=_h(offd, np.float64), rhs=_h(s.ls.GetResidual(), np.float64))
    del diag, offd
    assert s.factor()
    fdiag, foffd = s.prec.GetFactor()
    got.update(fdiag=_h(fdiag, np.float64), foffd=_h(foffd, np.float64))
    del fdiag, foffd
    r64 = s.solve("fp64")
    x64 = s.solution()
    sols = {}
    for mode in ("fp32f", "mixed"):
        s.assemble()
        assert s.factor()
        r = s.solve(mode, target_true=True)
        sols[mode] = (r, s.solution(), s.ls.true_residual())
    s.close()
    ref = _ref(oracle_runs, name)
    for k in ("rowptr", "colind", "diag", "offd", "rhs", "fdiag", "foffd"):
        assert got[k] == ref[k], f"{name}: {k} differs from the oracle's"
    xr = ref["x"]
    assert r64["converged"] and abs(r64["iter"] - ref["iter"]) <= 2, (r64, ref["iter"])
    assert _rel(x64, xr) <= 1e-6, _rel(x64, xr)
    for mode, (r, x, rel_true) in sols.items():
        assert r["converged"] and rel_true <= 1e-8, (mode, r, rel_true)
        assert _rel(x, xr) <= 1e-6, (mode, _rel(x, xr))
    print(f"{name}: oracle {ref['iter']} iterations ({ref['seconds']:.0f} s), GPU FP64 {r64['iter']} "
          f"(error {_rel(x64, xr):.1e}); " + ", ".join(
              f"{m} {r['iter']} iterations, true residual {t:.1e}, error {_rel(x, xr):.1e}"
              for m, (r, x, t) in sols.items()))


@pytest.mark.parametrize("name", ["serve2d_req12_poisson_376k", "serve2d_req48_solid_351k"])
def test_fullsize_served_request(gpu_ctx, oracle_runs, name):
    import oracle
    from delfem_gb300.serve import MODES, Server
    p = oracle.make_problem(SPECS[name])
    assert p.nnode >= 300_000
    out = {}
    for mode in MODES:
        with Server(gpu_ctx, mode=mode) as S:
            out[mode] = S.wait(S.submit(p))
    ref = _ref(oracle_runs, name)
    xr = ref["x"]
    for mode, r in out.items():
        assert r["status"] == 0 and 0.0 <= r["rel_true"] <= 1e-8, (mode, r)
        assert _rel(r["x"], xr) <= 1e-6, (mode, _rel(r["x"], xr))
    assert ref["iter"] - 2 <= out["fp64"]["iterations"] <= ref["iter"] + 8, (out["fp64"]["iterations"], ref["iter"])
    print(f"{name}: oracle {ref['iter']} iterations; " +
          ", ".join(f"{m} {r['iterations']} (error {_rel(r['x'], xr):.1e})" for m, r in out.items()))
