"""The CPU oracle (oracle/dfg_oracle.c) against the golden fixtures produced
by the reference itself: pattern, assembled matrix and right-hand side,
ILU(0) factor and the PCG result must be bit-identical."""
import numpy as np
import pytest

from conftest import bits, golden_files, load_golden


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
