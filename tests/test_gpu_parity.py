"""GPU parity through the C ABI against the reference (golden fixtures) and
the CPU oracle.

Bars (the parity tolerances, written per test):
  * assembled matrix and right-hand side: bit-identical to the reference
    (stronger than the 1e-12 relative-per-entry bar);
  * ILU(0) factor: bit-identical;
  * preconditioner apply: 1e-12 relative (FMA contraction in the sweeps);
  * PCG: iteration count within +-2 of the reference, solution within 1e-6
    relative L2 of the reference's, true relative residual <= 1e-8 for the
    mixed-precision solve (which targets the true residual).
"""
import numpy as np
import pytest

from conftest import bits, golden_files, load_golden

pytestmark = pytest.mark.gpu

GOLDEN_IDS = [p.rsplit("/", 1)[-1][:-4] for p in golden_files()]


def _solver(ctx, p):
    from delfem_gb300.solver import FESolve
    return FESolve(ctx, p)


@pytest.mark.parametrize("path", golden_files(), ids=GOLDEN_IDS)
def test_assembly_and_factor_bitexact(gpu_ctx, path):
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p)
    rowptr, colind = s.ls.pattern()
    assert np.array_equal(rowptr, ref["rowptr"]) and np.array_equal(colind, ref["colind"])
    norm = s.assemble()
    diag, offd = s.ls.GetMatrix()
    assert np.array_equal(bits(diag), bits(ref["diag"]))
    assert np.array_equal(bits(offd), bits(ref["offd"]))
    assert np.array_equal(bits(s.ls.GetResidual()), bits(ref["rhs"]))
    assert norm == pytest.approx(float(ref["norm_res"]), rel=1e-13)
    assert s.factor()
    fdiag, foffd = s.prec.GetFactor()
    assert np.array_equal(bits(fdiag), bits(ref["fdiag"]))
    assert np.array_equal(bits(foffd), bits(ref["foffd"]))
    s.close()


@pytest.mark.parametrize("path", golden_files(), ids=GOLDEN_IDS)
def test_precond_apply(gpu_ctx, oracle_lib, path):
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p)
    s.assemble()
    s.factor()
    n, b = p.nnode, p.b
    rhs = np.random.default_rng(1).standard_normal(n * b)
    s.ls.ReSizeTmpVecSolver(2)
    s.ls.SetVector(0, rhs)
    s.prec.SolvePrecond(s.ls, 0)
    z = s.ls.GetVector(0)
    dind = oracle_lib.diaind(ref["rowptr"], ref["colind"])
    zref = oracle_lib.precond(n, b, ref["rowptr"], ref["colind"], dind, ref["fdiag"], ref["foffd"], rhs)
    np.testing.assert_allclose(z, zref, rtol=1e-12, atol=1e-13 * np.abs(zref).max())
    s.close()


@pytest.mark.parametrize("path", golden_files(), ids=GOLDEN_IDS)
def test_pcg_fp64(gpu_ctx, oracle_lib, path):
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p)
    r = s.run("fp64", tol=1e-8, maxit=5000)
    assert r["converged"]
    assert abs(r["iter"] - int(ref["iter"])) <= 2
    x = s.solution()
    xr = ref["x"]
    assert np.linalg.norm(x - xr) <= 1e-6 * np.linalg.norm(xr)
    s.close()


@pytest.mark.parametrize("path", golden_files(), ids=GOLDEN_IDS)
def test_pcg_mixed(gpu_ctx, oracle_lib, path):
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p)
    r = s.run("mixed", tol=1e-8, maxit=20000)
    assert r["converged"], r
    assert r["conv"] <= 1e-8
    x = s.solution()
    assert s.ls.true_residual() <= 1e-8
    xr = ref["x"]
    assert np.linalg.norm(x - xr) <= 1e-6 * np.linalg.norm(xr)
    s.close()


@pytest.mark.parametrize("path", golden_files()[:5], ids=GOLDEN_IDS[:5])
def test_reference_control_flow_over_dropin(gpu_ctx, path):
    """The reference's Solve_PCG loop driving the GPU system through the
    ILinearSystemPreconditioner_Sol virtuals (the strict drop-in)."""
    from delfem_gb300 import linsys as L
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p)
    s.assemble()
    s.factor()
    ok, conv, it = L.Solve_PCG_reference_loop(1e-8, 5000, L.LinearSystemPreconditioner(s.ls, s.prec))
    assert ok
    assert abs(it - int(ref["iter"])) <= 2
    xr = ref["x"]
    assert np.linalg.norm(s.solution() - xr) <= 1e-6 * np.linalg.norm(xr)
    s.close()


def test_config1_poisson_128(gpu_ctx, oracle_lib):
    """The CPU-runnable configuration: 128x128 jittered Poisson, FP64 ILU(0)-PCG."""
    from delfem_gb300 import meshgen as mg
    p = mg.poisson2d_square(128)
    ref = oracle_lib.solve(p)
    s = _solver(gpu_ctx, p)
    r = s.run("fp64")
    assert r["converged"] and abs(r["iter"] - ref["iter"]) <= 2
    x = s.solution()
    assert np.linalg.norm(x - ref["x"]) <= 1e-6 * np.linalg.norm(ref["x"])
    diag, offd = s.ls.GetMatrix()
    assert np.array_equal(bits(diag), bits(ref["diag"])) and np.array_equal(bits(offd), bits(ref["offd"]))
    rm = s.run("mixed")
    assert rm["converged"] and s.ls.true_residual() <= 1e-8
    assert np.linalg.norm(s.solution() - ref["x"]) <= 1e-6 * np.linalg.norm(ref["x"])
    s.close()


@pytest.mark.parametrize("maker", ["solid2d", "solid3d"])
def test_medium_elasticity(gpu_ctx, oracle_lib, maker):
    from delfem_gb300 import meshgen as mg
    p = mg.solid2d_cantilever(80, 40, seed=21) if maker == "solid2d" else mg.solid3d_cube(10, seed=22)
    ref = oracle_lib.solve(p)
    s = _solver(gpu_ctx, p)
    r = s.run("fp64")
    assert r["converged"] and abs(r["iter"] - ref["iter"]) <= 2, (r, ref["iter"])
    assert np.linalg.norm(s.solution() - ref["x"]) <= 1e-6 * np.linalg.norm(ref["x"])
    rm = s.run("mixed")
    assert rm["converged"] and s.ls.true_residual() <= 1e-8
    assert np.linalg.norm(s.solution() - ref["x"]) <= 1e-6 * np.linalg.norm(ref["x"])
    s.close()


# ------------------------------------------------------------------ edge cases

def test_iteration_limit(gpu_ctx):
    from delfem_gb300 import meshgen as mg
    p, _ = load_golden(golden_files()[2])
    s = _solver(gpu_ctx, p)
    r = s.run("fp64", tol=1e-8, maxit=1)
    assert not r["converged"] and r["conv"] > 1e-8
    s.close()


def test_zero_rhs_returns_immediately(gpu_ctx):
    from delfem_gb300 import meshgen as mg
    p = mg.poisson2d_square(6)
    p.params = p.params.copy()
    p.params[1] = 0.0  # no source, homogeneous Dirichlet -> r0 = 0
    s = _solver(gpu_ctx, p)
    r = s.run("fp64")
    assert r["converged"] and r["iter"] == 0 and r["conv"] == 0.0
    assert not np.any(s.solution())
    s.close()


def test_singular_pivots_reported(gpu_ctx):
    from delfem_gb300 import meshgen as mg
    p = mg.poisson2d_square(6)
    s = _solver(gpu_ctx, p)
    s.assemble()
    diag, offd = s.ls.GetMatrix()
    s.ls.SetMatrix(np.zeros_like(diag), np.zeros_like(offd))
    assert s.factor() is False  # more than 10 zero pivots, as DoILUDecomp returns false
    s.close()


def test_fill_level_below_minus_one_rejected(gpu_ctx):
    """Levels >= -1 are the reference's (ILU(k), -1 = no limit); below is an error."""
    from delfem_gb300 import capi, linsys as L
    prec = L.PreconditionerILU(gpu_ctx)
    for lev in (0, 1, 7, -1):
        prec.SetFillInLevel(lev)
    with pytest.raises(capi.DfgError) as e:
        prec.SetFillInLevel(-3)
    assert e.value.status == capi.DFG_INVALID_ARGUMENT


def test_bad_pattern_rejected(gpu_ctx):
    from delfem_gb300 import capi, linsys as L
    with pytest.raises(capi.DfgError) as e:
        L.LinearSystemField(gpu_ctx, 3, 1, rowptr=np.array([0, 1, 1, 1]), colind=np.array([0]))
    assert e.value.status == capi.DFG_INVALID_ARGUMENT


def test_solution_is_deterministic(gpu_ctx):
    from delfem_gb300 import meshgen as mg
    p = mg.solid2d_cantilever(40, 20, seed=9)
    s = _solver(gpu_ctx, p)
    s.run("fp64")
    x1 = s.solution()
    s.run("fp64")
    x2 = s.solution()
    assert np.array_equal(bits(x1), bits(x2))
    s.close()


@pytest.mark.parametrize("path", golden_files(), ids=GOLDEN_IDS)
def test_pcg_fp32_factor(gpu_ctx, path):
    """FP32 factor and sweeps, FP64 SpMV and Krylov vectors, true residual enforced."""
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p)
    r = s.run("fp32f", tol=1e-8, maxit=5000, target_true=True)
    assert r["converged"] and r["conv"] <= 1e-8
    assert s.ls.true_residual() <= 1e-8
    # an FP32 factor is a slightly different preconditioner: a few more iterations
    assert r["iter"] <= 1.3 * int(ref["iter"]) + 6
    xr = ref["x"]
    assert np.linalg.norm(s.solution() - xr) <= 1e-6 * np.linalg.norm(xr)
    s.close()


def test_fp64_true_residual_target(gpu_ctx, oracle_lib):
    from delfem_gb300 import meshgen as mg
    p = mg.solid2d_cantilever(60, 30, seed=31)
    s = _solver(gpu_ctx, p)
    r = s.run("fp64", target_true=True)
    assert r["converged"] and r["conv"] <= 1e-8 and s.ls.true_residual() <= 1e-8
    s.close()


def test_bounded_wait_times_out_and_context_stays_usable(gpu_ctx):
    """A device wait on a value nothing writes gives up after its budget,
    reports DFG_TIMEOUT with the wait site, and the context keeps working."""
    import ctypes
    import time
    from delfem_gb300 import capi
    from delfem_gb300 import meshgen as mg
    site = ctypes.c_int(0)
    t0 = time.perf_counter()
    st = capi.lib().dfg_selftest_wait_timeout(gpu_ctx.h, ctypes.byref(site))
    waited = time.perf_counter() - t0
    assert st == capi.DFG_TIMEOUT and site.value == 3
    assert 0.5 < waited < 30.0
    assert b"timed out" in capi.lib().dfg_last_error(gpu_ctx.h)
    s = _solver(gpu_ctx, mg.poisson2d_square(8, seed=3))
    r = s.run("fp64")
    assert r["converged"]
    s.close()
