"""ILU(k) (CPreconditioner_ILU::SetFillInLevel(k), k != 0) on the GPU against
the reference: fill pattern and factor bit-identical to the reference's
(tests/golden/iluk/, produced by the reference itself), substitutions and
PCG within the same bars as ILU(0).  Larger meshes are checked against the
oracle, which is pinned to the reference at these levels."""
import numpy as np
import pytest

from conftest import bits, golden_iluk_files, load_golden

pytestmark = pytest.mark.gpu

IDS = [p.rsplit("/", 1)[-1][:-4] for p in golden_iluk_files()]


def _solver(ctx, p, lev):
    from delfem_gb300.solver import FESolve
    return FESolve(ctx, p, fill_level=lev)


@pytest.mark.parametrize("path", golden_iluk_files(), ids=IDS)
def test_iluk_pattern_and_factor_bitexact(gpu_ctx, path):
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p, int(ref["fill_level"]))
    rp, ci = s.prec.GetPattern()
    assert np.array_equal(rp, ref["rowptr_f"]) and np.array_equal(ci, ref["colind_f"])
    s.assemble()
    assert s.factor()
    fdiag, foffd = s.prec.GetFactor()
    assert np.array_equal(bits(fdiag), bits(ref["fdiag"]))
    assert np.array_equal(bits(foffd), bits(ref["foffd"]))
    s.close()


@pytest.mark.parametrize("path", golden_iluk_files(), ids=IDS)
def test_iluk_precond_apply(gpu_ctx, oracle_lib, path):
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p, int(ref["fill_level"]))
    s.assemble()
    s.factor()
    n, b = p.nnode, p.b
    rhs = np.random.default_rng(2).standard_normal(n * b)
    s.ls.ReSizeTmpVecSolver(2)
    s.ls.SetVector(0, rhs)
    s.prec.SolvePrecond(s.ls, 0)
    z = s.ls.GetVector(0)
    rp, ci = ref["rowptr_f"], ref["colind_f"]
    zref = oracle_lib.precond(n, b, rp, ci, oracle_lib.diaind(rp, ci), ref["fdiag"], ref["foffd"], rhs)
    np.testing.assert_allclose(z, zref, rtol=1e-12, atol=1e-13 * np.abs(zref).max())
    s.close()


@pytest.mark.parametrize("path", golden_iluk_files(), ids=IDS)
def test_iluk_pcg_fp64(gpu_ctx, path):
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p, int(ref["fill_level"]))
    r = s.run("fp64", tol=1e-8, maxit=5000)
    assert r["converged"]
    assert abs(r["iter"] - int(ref["iter"])) <= 2
    xr = ref["x"]
    assert np.linalg.norm(s.solution() - xr) <= 1e-6 * np.linalg.norm(xr)
    s.close()


@pytest.mark.parametrize("mode", ["fp32f", "mixed"])
@pytest.mark.parametrize("path", golden_iluk_files()[:4], ids=IDS[:4])
def test_iluk_precision_forms(gpu_ctx, path, mode):
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p, int(ref["fill_level"]))
    r = s.run(mode, tol=1e-8, maxit=20000, target_true=True)
    assert r["converged"], r
    assert s.ls.true_residual() <= 1e-8
    xr = ref["x"]
    assert np.linalg.norm(s.solution() - xr) <= 1e-6 * np.linalg.norm(xr)
    s.close()


@pytest.mark.parametrize("path", golden_iluk_files()[:3], ids=IDS[:3])
def test_iluk_reference_control_flow_over_dropin(gpu_ctx, path):
    from delfem_gb300 import linsys as L
    p, ref = load_golden(path)
    s = _solver(gpu_ctx, p, int(ref["fill_level"]))
    s.assemble()
    s.factor()
    ok, conv, it = L.Solve_PCG_reference_loop(1e-8, 5000, L.LinearSystemPreconditioner(s.ls, s.prec))
    assert ok and abs(it - int(ref["iter"])) <= 2
    xr = ref["x"]
    assert np.linalg.norm(s.solution() - xr) <= 1e-6 * np.linalg.norm(xr)
    s.close()


@pytest.mark.parametrize("kind,lev", [("solid2d", 1), ("poisson3d", 2), ("solid3d", 1), ("poisson2d", -1)])
def test_iluk_larger_meshes_vs_oracle(gpu_ctx, oracle_lib, kind, lev):
    from delfem_gb300 import meshgen as mg
    p = {"solid2d": lambda: mg.solid2d_cantilever(120, 60, seed=31, coef_sigma=0.5),
         "poisson3d": lambda: mg.poisson3d_cube(14, seed=32, coef_sigma=1.0),
         "solid3d": lambda: mg.solid3d_cube(8, seed=33, coef_sigma=1.0),
         "poisson2d": lambda: mg.poisson2d_square(24, seed=34)}[kind]()
    ref = oracle_lib.solve(p, fill_level=lev)
    s = _solver(gpu_ctx, p, lev)
    rp, ci = s.prec.GetPattern()
    assert np.array_equal(rp, ref["rowptr_f"]) and np.array_equal(ci, ref["colind_f"])
    r = s.run("fp64", tol=1e-8, maxit=5000)
    fdiag, foffd = s.prec.GetFactor()
    assert np.array_equal(bits(fdiag), bits(ref["fdiag"])) and np.array_equal(bits(foffd), bits(ref["foffd"]))
    assert r["converged"] and abs(r["iter"] - ref["iter"]) <= 2, (r["iter"], ref["iter"])
    xr = ref["x"]
    assert np.linalg.norm(s.solution() - xr) <= 1e-6 * np.linalg.norm(xr)
    s.close()


def test_fill_level_switch_and_reject(gpu_ctx):
    """The level takes effect at the next symbolic set-up; < -1 is rejected."""
    from delfem_gb300 import capi
    from delfem_gb300 import meshgen as mg
    p = mg.solid2d_cantilever(20, 8, seed=35)
    s = _solver(gpu_ctx, p, 1)
    nnz1 = s.prec.GetPattern()[1].size
    assert nnz1 > s.ls.nnz
    s.prec.SetFillInLevel(0)
    s.prec.SetLinearSystem(s.ls)
    assert np.array_equal(s.prec.GetPattern()[1], s.ls.pattern()[1])
    r0 = s.run("fp64")
    s.prec.SetFillInLevel(1)
    s.prec.SetLinearSystem(s.ls)
    assert s.prec.GetPattern()[1].size == nnz1
    r1 = s.run("fp64")
    assert r0["converged"] and r1["converged"] and r1["iter"] < r0["iter"]
    with pytest.raises(capi.DfgError) as e:
        s.prec.SetFillInLevel(-2)
    assert e.value.status == capi.DFG_INVALID_ARGUMENT
    s.close()
