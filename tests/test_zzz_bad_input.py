"""Bad input on the GPU, made on the host: an equation on a mesh or block
length it does not take, and a NaN element coefficient.  Each case must end
in the status the reference's behaviour implies and leave the context
usable.  This file runs after the rest of the GPU suite."""
import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu


def test_equation_mesh_mismatch_rejected(gpu_ctx, oracle_lib):
    """An equation on a mesh or block length it does not take is rejected
    before anything is written, and the system stays usable: diffusion on
    tetrahedra (the CLinearSystem_Field overload of AddLinSys_Diffusion takes
    triangles only, src/femeqn/eqn_diffusion.cpp:348-398, and reports
    anything else as not implemented), 2D elasticity on a scalar system, 3D
    elasticity on a triangle mesh."""
    from delfem_gb300 import capi, linsys as L, meshgen as mg
    p = mg.poisson3d_cube(4, seed=81)
    ls = L.LinearSystemField(gpu_ctx, p.nnode, 1, conn=p.conn)
    try:
        ls.set_mesh(p.coords, p.conn)
        ls.InitializeMarge()
        for call in (lambda: L.AddLinSys_Diffusion(0.1, 0.5, ls, 1.0, 1.0, 1.0),
                     lambda: L.AddLinSys_LinearSolid2D_Static(ls, 1.0, 1.0, 0.0, 0.0, 0.0)):
            with pytest.raises(capi.DfgError) as e:
                call()
            assert e.value.status == capi.DFG_INVALID_ARGUMENT
        L.AddLinSys_Poisson(ls, float(p.params[0]), float(p.params[1]))
        rp, ci = oracle_lib.pattern(p.nnode, p.conn)
        diag, offd, res = oracle_lib.assemble(p, rp, ci)
        gd, go = ls.GetMatrix()
        assert np.array_equal(bits(gd), bits(diag)) and np.array_equal(bits(go), bits(offd))
        assert np.array_equal(bits(ls.GetResidual()), bits(res))
    finally:
        ls.close()
    q = mg.solid2d_cantilever(6, 3, seed=82)
    ls = L.LinearSystemField(gpu_ctx, q.nnode, 3, conn=q.conn)
    try:
        ls.set_mesh(q.coords, q.conn)
        ls.InitializeMarge()
        with pytest.raises(capi.DfgError) as e:
            L.AddLinSys_LinearSolid3D_Static(ls, 1.0, 1.0, 0.0, 0.0, 0.0, 0.0)
        assert e.value.status == capi.DFG_INVALID_ARGUMENT
    finally:
        ls.close()


@pytest.mark.parametrize("kind,where", [("poisson2d", "first"), ("poisson2d", "last"), ("solid3d", "first"),
                                        ("solid3d", "last")])
def test_nan_coefficient(gpu_ctx, oracle_lib, kind, where):
    """Bad data made on the host: one NaN element coefficient.  It reaches the
    same matrix entries as in the reference (NaN positions compared, every
    other entry bit-exact; NaN payloads are the platform's).  A NaN pivot is
    singular (fabs(NaN) > 1e-30 is false, matdiafrac_blkcrs.cpp:885-895), so
    the factor fails exactly when DoILUDecomp does (more than 10: a NaN early
    in the numbering spreads to later rows); when it does not, the solve
    stops with DFG_NAN_DETECTED rather than iterating to its limit.  The
    context stays usable."""
    from delfem_gb300 import capi, linsys as L, meshgen as mg
    from delfem_gb300.solver import FESolve
    p = (mg.poisson2d_square(16, seed=91, coef_sigma=0.5) if kind == "poisson2d"
         else mg.solid3d_cube(4, seed=93, coef_sigma=0.5))
    p.coef[0 if where == "first" else p.nelem - 1] = np.nan
    ref = oracle_lib.solve(p, stop_after_ilu=True)
    s = FESolve(gpu_ctx, p)
    try:
        assert np.isnan(s.assemble())
        gd, go = s.ls.GetMatrix()
        # (the Dirichlet rows and columns can clear every NaN off-diagonal block)
        for g, r, some in ((gd, ref["diag"], True), (go, ref["offd"], False), (s.ls.GetResidual(), ref["rhs"], True)):
            m = np.isnan(r)
            assert (m.any() or not some) and np.array_equal(np.isnan(g), m)
            assert np.array_equal(bits(g[~m]), bits(r[~m]))
        ok = s.factor()
        assert ok == (ref["ilu_rc"] >= 0), ref["ilu_rc"]
        if ok:
            fd, _ = s.prec.GetFactor()
            assert np.array_equal(np.isnan(fd), np.isnan(ref["fdiag"]))
            with pytest.raises(capi.DfgError) as e:
                L.Solve_PCG(1e-8, 1000, s.ls, s.prec)
            assert e.value.status == capi.DFG_NAN_DETECTED
    finally:
        s.close()
    q = mg.poisson2d_square(12, seed=94)
    rq = oracle_lib.solve(q)
    s = FESolve(gpu_ctx, q)
    try:
        r = s.run("fp64")
        assert r["converged"] and abs(r["iter"] - rq["iter"]) <= 2
        assert np.linalg.norm(s.solution() - rq["x"]) <= 1e-6 * np.linalg.norm(rq["x"])
    finally:
        s.close()
