"""Preconditioned BiCGSTAB (LsSol::Solve_PBiCGSTAB) on the GPU through the C
ABI against the reference: the fixtures in tests/golden/bicgstab/ come from
the reference itself (iterations, ratio, solution; its early return on a zero
right-hand side and its untouched ratio at the iteration limit), and
non-symmetric systems are checked against the oracle, which is pinned to the
reference bit for bit.  Bars: iterations within +-2, solution within 1e-6
relative L2, true relative residual within 10x the tolerance."""
import numpy as np
import pytest

from conftest import bits, golden_bicgstab_files, load_golden

pytestmark = pytest.mark.gpu

IDS = [p.rsplit("/", 1)[-1][:-4] for p in golden_bicgstab_files()]


def _setup(ctx, p, lev):
    from delfem_gb300.solver import FESolve
    s = FESolve(ctx, p, fill_level=lev)
    s.assemble()
    assert s.factor()
    return s


def _rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


@pytest.mark.parametrize("path", golden_bicgstab_files(), ids=IDS)
def test_bicgstab_matches_reference(gpu_ctx, path):
    from delfem_gb300 import linsys as L
    p, ref = load_golden(path)
    s = _setup(gpu_ctx, p, int(ref["fill_level"]))
    rhs = s.ls.GetResidual().copy()
    ok, conv, it = L.Solve_PBiCGSTAB(p.tol, p.maxit, s.ls, s.prec)
    x = s.solution()
    if int(ref["iter"]) == 0:  # zero right-hand side: immediate return, x untouched
        assert ok and it == 0 and conv == float(ref["conv"]) and not np.any(x)
    elif int(ref["iter"]) == p.maxit:  # limit reached: ratio as given, iteration = limit
        assert not ok and it == p.maxit and conv == p.tol
        assert _rel(x, ref["x"]) <= 1e-6
    else:
        assert ok and conv < p.tol
        assert abs(it - int(ref["iter"])) <= 2, (it, int(ref["iter"]))
        assert _rel(x, ref["x"]) <= 1e-6
        assert s.ls.true_residual(rhs) <= 10 * p.tol
    s.close()


@pytest.mark.parametrize("path", golden_bicgstab_files()[:3], ids=IDS[:3])
def test_bicgstab_reference_control_flow_over_dropin(gpu_ctx, path):
    """The reference's Solve_PBiCGSTAB loop over the drop-in virtuals."""
    from delfem_gb300 import linsys as L
    p, ref = load_golden(path)
    s = _setup(gpu_ctx, p, int(ref["fill_level"]))
    ok, conv, it = L.Solve_PBiCGSTAB_reference_loop(p.tol, p.maxit, L.LinearSystemPreconditioner(s.ls, s.prec))
    assert ok and abs(it - int(ref["iter"])) <= 2
    assert _rel(s.solution(), ref["x"]) <= 1e-6
    s.close()


def _skew(out, c, seed):
    """The assembled matrix plus a skew-symmetric part on its pattern (a
    convection-like term): A_ij += c w_ij, A_ji -= c w_ij, rows and columns of
    Dirichlet DOFs left as the finalize made them."""
    n, b = out["n"], out["b"]
    bs = b * b
    rp, ci = out["rowptr"], out["colind"]
    offd = out["offd"].reshape(-1, b, b).copy()
    rng = np.random.default_rng(seed)
    scale = np.abs(offd).max()
    fixed = np.zeros(n * b, bool)
    for i in range(n):
        for d in range(b):
            blk = out["diag"][i * bs + d * b + d]
            row = offd[rp[i]:rp[i + 1], d, :]
            fixed[i * b + d] = blk == 1.0 and not np.any(row)
    slot = {}
    for i in range(n):
        for c_ in range(rp[i], rp[i + 1]):
            slot[(i, int(ci[c_]))] = c_
    for i in range(n):
        for c_ in range(rp[i], rp[i + 1]):
            j = int(ci[c_])
            if j <= i:
                continue
            w = c * scale * rng.uniform(-1, 1, (b, b))
            t = slot[(j, i)]
            for d in range(b):
                for e in range(b):
                    if fixed[i * b + d] or fixed[j * b + e]:
                        continue
                    offd[c_, d, e] += w[d, e]
                    offd[t, e, d] -= w[d, e]
    return offd.reshape(-1)


@pytest.mark.parametrize("kind,lev", [("poisson2d", 0), ("solid2d", 0), ("solid2d", 1), ("poisson3d", 0)])
def test_bicgstab_nonsymmetric_vs_oracle(gpu_ctx, oracle_lib, kind, lev):
    from delfem_gb300 import linsys as L
    from delfem_gb300 import meshgen as mg
    p = {"poisson2d": lambda: mg.poisson2d_square(40, seed=41, coef_sigma=0.5),
         "solid2d": lambda: mg.solid2d_cantilever(60, 20, seed=42, coef_sigma=0.5),
         "poisson3d": lambda: mg.poisson3d_cube(10, seed=43)}[kind]()
    out = oracle_lib.solve(p, stop_after_ilu=True, fill_level=lev)
    offd_ns = _skew(out, 0.05, seed=44)
    fdiag, foffd, rc = oracle_lib.factor(out, out["diag"], offd_ns)
    assert rc >= 0
    ref = oracle_lib.bicgstab(dict(out, fdiag=fdiag, foffd=foffd), 1e-8, 5000, offd=offd_ns)
    assert ref["converged"]
    s = _setup(gpu_ctx, p, lev)
    s.ls.SetMatrix(out["diag"], offd_ns)
    assert s.factor()
    gd, go = s.prec.GetFactor()
    assert np.array_equal(bits(gd), bits(fdiag)) and np.array_equal(bits(go), bits(foffd))
    ok, conv, it = L.Solve_PBiCGSTAB(1e-8, 5000, s.ls, s.prec)
    assert ok and conv < 1e-8
    assert abs(it - ref["iter"]) <= 2, (it, ref["iter"])
    x = s.solution()
    assert _rel(x, ref["x"]) <= 1e-6
    Ax = oracle_lib.matvec(out["n"], out["b"], out["rowptr"], out["colind"], out["diag"], offd_ns, x)
    assert np.linalg.norm(out["rhs"] - Ax) <= 1e-7 * np.linalg.norm(out["rhs"])
    s.close()


def test_bicgstab_rejects_fp32_modes_and_is_repeatable(gpu_ctx):
    from delfem_gb300 import capi
    from delfem_gb300 import linsys as L
    from delfem_gb300 import meshgen as mg
    p = mg.solid2d_cantilever(30, 12, seed=45)
    s = _setup(gpu_ctx, p, 0)
    rhs = s.ls.GetResidual().copy()
    for mode in ("mixed", "fp32f"):
        with pytest.raises(capi.DfgError) as e:
            L.Solve_PBiCGSTAB(1e-8, 100, s.ls, s.prec, mode)
        assert e.value.status == capi.DFG_INVALID_ARGUMENT
    ok1, c1, it1 = L.Solve_PBiCGSTAB(1e-8, 1000, s.ls, s.prec)
    x1 = s.solution()
    s.ls.SetVector(-1, rhs)
    ok2, c2, it2 = L.Solve_PBiCGSTAB(1e-8, 1000, s.ls, s.prec)
    assert ok1 and ok2 and it1 == it2 and c1 == c2
    assert np.array_equal(bits(x1), bits(s.solution()))
    s.close()
