"""The three sweep schedules (dfg_precond_set_sweep_mode: 1 ranged, 2
level-scheduled, 3 one CTA) against the oracle: the preconditioner apply to
1e-12, FP64 PCG within +-2 iterations and 1e-6 of the oracle's solution, the
precision forms to a true residual of 1e-8, BiCGSTAB, and ILU(1) on the
level and one-CTA schedules; the timed choice picks one kind per direction."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(kind):
    from delfem_gb300 import meshgen as mg
    return {"poisson2d": lambda: mg.poisson2d_square(60, seed=71, coef_sigma=0.5),
            "solid2d": lambda: mg.solid2d_cantilever(50, 20, seed=72, coef_sigma=0.5),
            "poisson3d": lambda: mg.poisson3d_cube(12, seed=73, coef_sigma=1.0),
            "solid3d": lambda: mg.solid3d_cube(8, seed=74, coef_sigma=1.0)}[kind]()


@pytest.mark.parametrize("mode", [1, 2, 3])
@pytest.mark.parametrize("kind", ["poisson2d", "solid2d", "poisson3d", "solid3d"])
def test_sweep_modes(gpu_ctx, oracle_lib, kind, mode):
    from delfem_gb300 import linsys as L
    from delfem_gb300.solver import FESolve
    p = _problem(kind)
    ref = oracle_lib.solve(p)
    s = FESolve(gpu_ctx, p, sweep_mode=mode)
    try:
        assert s.prec.GetSweepMode() == (mode, mode)
        s.assemble()
        assert s.factor()
        n, b = p.nnode, p.b
        rhs = np.random.default_rng(3).standard_normal(n * b)
        s.ls.ReSizeTmpVecSolver(1)
        s.ls.SetVector(0, rhs)
        s.prec.SolvePrecond(s.ls, 0)
        z = s.ls.GetVector(0)
        zref = oracle_lib.precond(n, b, ref["rowptr"], ref["colind"], ref["diaind"], ref["fdiag"], ref["foffd"], rhs)
        np.testing.assert_allclose(z, zref, rtol=1e-12, atol=1e-13 * np.abs(zref).max())
        r = s.run("fp64")
        assert r["converged"] and abs(r["iter"] - ref["iter"]) <= 2, (r["iter"], ref["iter"])
        xr = ref["x"]
        assert np.linalg.norm(s.solution() - xr) <= 1e-6 * np.linalg.norm(xr)
        for mode_p in ("fp32f", "mixed"):
            rm = s.run(mode_p, target_true=True)
            assert rm["converged"] and s.ls.true_residual() <= 1e-8, (mode_p, rm)
            assert np.linalg.norm(s.solution() - xr) <= 1e-6 * np.linalg.norm(xr)
        s.assemble()
        s.factor()
        ok, conv, it = L.Solve_PBiCGSTAB(1e-8, 5000, s.ls, s.prec)
        assert ok and np.linalg.norm(s.solution() - xr) <= 1e-6 * np.linalg.norm(xr)
    finally:
        s.close()


@pytest.mark.parametrize("mode", [2, 3])
def test_schedule_with_fill_in(gpu_ctx, oracle_lib, mode):
    from delfem_gb300.solver import FESolve
    p = _problem("solid3d")
    ref = oracle_lib.solve(p, fill_level=1)
    s = FESolve(gpu_ctx, p, fill_level=1, sweep_mode=mode)
    try:
        r = s.run("fp64")
        assert r["converged"] and abs(r["iter"] - ref["iter"]) <= 2
        assert np.linalg.norm(s.solution() - ref["x"]) <= 1e-6 * np.linalg.norm(ref["x"])
        rm = s.run("fp32f", target_true=True)
        assert rm["converged"] and s.ls.true_residual() <= 1e-8
    finally:
        s.close()


def test_timed_choice_and_bad_mode(gpu_ctx):
    from delfem_gb300 import capi
    from delfem_gb300.solver import FESolve
    s = FESolve(gpu_ctx, _problem("poisson3d"))
    try:
        f, b = s.prec.GetSweepMode()
        assert f in (1, 2, 3) and b in (1, 2, 3)
        solo = s.prec.GetSoloTiming()
        assert all(t > 0 for t in solo) or all(t == -1 for t in solo)
        with pytest.raises(capi.DfgError) as e:
            s.prec.SetSweepMode(4)
        assert e.value.status == capi.DFG_INVALID_ARGUMENT
    finally:
        s.close()
