"""Mesh input and field write-back on the GPU: a mesh written to and read
from a GiD file solves exactly as the oracle's run on the original arrays,
and UpdateValueOfField on the resident field (dfg_system_update_field) adds
the update bit for bit as the reference's AddValueToNodeSegment(.., 1.0)
does, so that the next assembly sees it without a host round trip."""
import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["solid2d", "poisson3d"])
def test_solve_on_mesh_read_from_file(gpu_ctx, oracle_lib, tmp_path, kind):
    from delfem_gb300 import meshgen as mg
    from delfem_gb300.solver import FESolve
    rng = np.random.default_rng(11)
    if kind == "solid2d":
        co, cn = mg.tri_grid(40, 16, 2.5, 1.0, 0.2, rng)
        k = mg.SOLID2D
    else:
        co, cn = mg.tet_grid(8, 7, 6, jitter=0.15, rng=rng)
        k = mg.POISSON3D
    path = str(tmp_path / "m.msh")
    mg.write_gid_msh(path, co, cn)
    rco, rcn = mg.read_gid_msh(path)
    p = mg.mesh_problem(k, rco, rcn, seed=2, coef_sigma=0.5)
    ref = oracle_lib.solve(p)
    s = FESolve(gpu_ctx, p)
    r = s.run("fp64")
    diag, offd = s.ls.GetMatrix()
    assert np.array_equal(bits(diag), bits(ref["diag"])) and np.array_equal(bits(offd), bits(ref["offd"]))
    assert r["converged"] and abs(r["iter"] - ref["iter"]) <= 2
    assert np.linalg.norm(s.solution() - ref["x"]) <= 1e-6 * np.linalg.norm(ref["x"])
    s.close()


def test_update_field_on_device(gpu_ctx, oracle_lib):
    """Static solve, field += update on the device, re-assembly with the new
    field (residual f - K u, now near zero), second solve, update again."""
    from delfem_gb300 import meshgen as mg
    from delfem_gb300.solver import FESolve
    p = mg.solid2d_cantilever(30, 12, seed=7, coef_sigma=0.5)
    s = FESolve(gpu_ctx, p)
    u0, v0 = s.ls.get_field()
    assert not np.any(u0) and not np.any(v0)
    norm1 = s.assemble()
    s.factor()
    r1 = s.solve("fp64")
    x1 = s.solution()
    s.ls.UpdateValueOfField(0)
    u1, _ = s.ls.get_field()
    assert np.array_equal(bits(u1), bits(0.0 + x1))
    # the oracle's assembly with the same field gives the same residual
    p1 = mg.Problem(p.kind, p.coords, p.conn, p.params, p.bcflag, coef=p.coef, load=p.load, u=u1)
    ref = oracle_lib.solve(p1, stop_after_ilu=True)
    norm2 = s.assemble()
    assert np.array_equal(bits(s.ls.GetResidual()), bits(ref["rhs"]))
    assert norm2 == pytest.approx(float(ref["norm_res"]), rel=1e-13)
    assert norm2 <= 1e-7 * norm1
    s.factor()
    s.solve("fp64")
    x2 = s.solution()
    s.ls.UpdateValueOfField(0)
    u2, _ = s.ls.get_field()
    assert np.array_equal(bits(u2), bits(u1 + x2))
    assert np.linalg.norm(x2) <= 1e-6 * np.linalg.norm(x1)
    assert r1["converged"]
    s.close()


def test_update_velocity_and_reject_bad_fdt(gpu_ctx):
    from delfem_gb300 import capi
    from delfem_gb300 import meshgen as mg
    from delfem_gb300.solver import FESolve
    p = mg.diffusion2d_square(10, seed=8)
    s = FESolve(gpu_ctx, p)
    s.run("fp64")
    x = s.solution()
    u0, v0 = s.ls.get_field()
    s.ls.UpdateValueOfField(1)
    u1, v1 = s.ls.get_field()
    assert np.array_equal(bits(u1), bits(u0)) and np.array_equal(bits(v1), bits(v0 + x))
    with pytest.raises(capi.DfgError) as e:
        s.ls.UpdateValueOfField(2)
    assert e.value.status == capi.DFG_INVALID_ARGUMENT
    s.close()
