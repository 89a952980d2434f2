"""The CPU oracle (oracle/dfg_oracle.c) against the golden fixtures produced
by the reference itself: pattern, assembled matrix and right-hand side,
ILU(0) factor and the PCG result must be bit-identical."""
import numpy as np
import pytest

from conftest import bits, golden_bicgstab_files, golden_files, golden_iluk_files, load_golden


@pytest.mark.parametrize("path", golden_files(), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_oracle_matches_reference(path, oracle_lib):
    p, ref = load_golden(path)
    out = oracle_lib.solve(p)
    assert np.array_equal(out["rowptr"], ref["rowptr"])
    assert np.array_equal(out["colind"], ref["colind"])
    for k in ("diag", "offd", "rhs", "fdiag", "foffd", "x"):
        assert np.array_equal(bits(out[k]), bits(ref[k])), k
    assert out["iter"] == int(ref["iter"])
    assert out["conv"] == float(ref["conv"])
    assert out["norm_res"] == float(ref["norm_res"])
    assert out["converged"] == bool(ref["converged"])


def test_golden_fixtures_present():
    assert len(golden_files()) >= 9


@pytest.mark.parametrize("path", golden_files()[:3], ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_reference_solution_meets_tolerance(path, oracle_lib):
    p, ref = load_golden(path)
    out = oracle_lib.solve(p, stop_after_ilu=True)
    rel = oracle_lib.true_residual(out, ref["x"])
    assert rel < 1e-7


@pytest.mark.parametrize("path", golden_iluk_files(), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_oracle_iluk_matches_reference(path, oracle_lib):
    """ILU(k): the fill pattern (AddFracPtn), the factor on it and the PCG
    result are bit-identical to the reference's at the fixture's level."""
    p, ref = load_golden(path)
    lev = int(ref["fill_level"])
    out = oracle_lib.solve(p, fill_level=lev)
    assert np.array_equal(out["rowptr_f"], ref["rowptr_f"])
    assert np.array_equal(out["colind_f"], ref["colind_f"])
    for k in ("diag", "offd", "rhs", "fdiag", "foffd", "x"):
        assert np.array_equal(bits(out[k]), bits(ref[k])), k
    assert out["iter"] == int(ref["iter"]) and out["conv"] == float(ref["conv"])


def test_iluk_fixtures_cover_levels():
    levs = sorted(int(load_golden(f)[1]["fill_level"]) for f in golden_iluk_files())
    assert levs[0] == -1 and 1 in levs and 2 in levs and 3 in levs


def test_iluk_pattern_properties(oracle_lib):
    """Level 0 leaves the pattern as it is; every level keeps A's pattern;
    the unlimited level gives the complete fill of natural-order LU."""
    from delfem_gb300 import meshgen as mg
    p = mg.poisson2d_square(9, seed=3)
    rp, ci = oracle_lib.pattern(p.nnode, p.conn)
    r0, c0 = oracle_lib.ilu_pattern(rp, ci, 0)
    assert np.array_equal(r0, rp) and np.array_equal(c0, ci)
    n = rp.size - 1
    for lev in (1, 2, 5, -1):
        rf, cf = oracle_lib.ilu_pattern(rp, ci, lev)
        for i in range(n):
            assert set(ci[rp[i]:rp[i + 1]]) <= set(cf[rf[i]:rf[i + 1]])
            assert np.all(np.diff(cf[rf[i]:rf[i + 1]]) > 0) and i not in set(cf[rf[i]:rf[i + 1]])
    # complete LU fill of the structurally symmetric pattern: row i holds every
    # column j > i up to its last original neighbour's reach (the profile)
    rf, cf = oracle_lib.ilu_pattern(rp, ci, -1)
    dense = np.zeros((n, n), bool)
    for i in range(n):
        dense[i, ci[rp[i]:rp[i + 1]]] = True
    for k in range(n):  # symbolic Gaussian elimination
        lower = np.nonzero(dense[k + 1:, k])[0] + k + 1
        upper = np.nonzero(dense[k, k + 1:])[0] + k + 1
        for i in lower:
            dense[i, upper] = True
    np.fill_diagonal(dense, False)
    for i in range(n):
        assert np.array_equal(cf[rf[i]:rf[i + 1]], np.nonzero(dense[i])[0]), i


@pytest.mark.parametrize("path", golden_bicgstab_files(), ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_oracle_bicgstab_matches_reference(path, oracle_lib):
    """Solve_PBiCGSTAB: solution, ratio and iteration count bit-identical to
    the reference's, including its early return on a zero right-hand side and
    its untouched ratio when the iteration limit is reached."""
    p, ref = load_golden(path)
    assert str(ref["solver"]) == "bicgstab"
    out = oracle_lib.solve(p, fill_level=int(ref["fill_level"]), solver="bicgstab")
    assert np.array_equal(bits(out["x"]), bits(ref["x"]))
    assert out["iter"] == int(ref["iter"]) and out["conv"] == float(ref["conv"])
    if out["iter"] == p.maxit:
        assert not out["converged"] and out["conv"] == p.tol  # the reference returns true here
    else:
        assert out["converged"]


def test_bicgstab_fixtures_cover_quirks():
    refs = [load_golden(f) for f in golden_bicgstab_files()]
    assert any(int(r["iter"]) == 0 and float(r["conv"]) == 0.0 for _, r in refs)
    assert any(int(r["iter"]) == p.maxit for p, r in refs)
    assert any(int(r["fill_level"]) == 1 for _, r in refs)
