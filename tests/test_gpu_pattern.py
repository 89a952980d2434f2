"""Pattern and assembly gather map built on the device (k_pattern.cu), used
by dfg_system_create_from_elements and dfg_system_set_mesh.  They must give
the host builders' results bit for bit: the pattern equals the oracle's
(MakePattern_FEM + AddPattern) and the assembled matrix and right-hand side
equal the oracle's (the element order of Mearge).  Nodes whose lists exceed
a thread's bound are built on the host; blocks outside a given pattern are
skipped as Mearge skips them; a failed set_mesh leaves the previous mesh."""
import numpy as np
import pytest

from conftest import bits

pytestmark = pytest.mark.gpu


def _check_assembly(ctx, oracle_lib, p, rowptr=None, colind=None):
    from delfem_gb300 import linsys as L
    from delfem_gb300.solver import FESolve
    if rowptr is None:
        # the whole path: pattern, then the matrix and right-hand side after
        # the Dirichlet finalize against the oracle's
        s = FESolve(ctx, p)
        try:
            rp, ci = s.ls.pattern()
            ref = oracle_lib.solve(p, stop_after_ilu=True)
            assert np.array_equal(rp, ref["rowptr"]) and np.array_equal(ci, ref["colind"])
            s.assemble()
            gd, go = s.ls.GetMatrix()
            assert np.array_equal(bits(gd), bits(ref["diag"])) and np.array_equal(bits(go), bits(ref["offd"]))
            assert np.array_equal(bits(s.ls.GetResidual()), bits(ref["rhs"]))
        finally:
            s.close()
        return
    # a given pattern: the element assembly alone (before loads and Dirichlet)
    rr, rc = rowptr, colind
    ls = L.LinearSystemField(ctx, p.nnode, p.b, rowptr=rr, colind=rc)
    try:
        ls.set_mesh(p.coords, p.conn)
        if p.coef is not None:
            ls.set_coef(p.coef)
        ls.InitializeMarge()
        P = [float(x) for x in p.params]
        if p.kind == 4:
            L.AddLinSys_LinearSolid2D_Static(ls, P[0], P[1], P[2], P[3], P[4])
        else:
            L.AddLinSys_Poisson(ls, P[0], P[1])
        diag, offd, res = oracle_lib.assemble(p, rr, rc)
        gd, go = ls.GetMatrix()
        assert np.array_equal(bits(gd), bits(diag)) and np.array_equal(bits(go), bits(offd))
        assert np.array_equal(bits(ls.GetResidual()), bits(res))
    finally:
        ls.close()


@pytest.mark.parametrize("kind", ["poisson2d", "solid2d", "poisson3d", "solid3d"])
def test_device_pattern_and_gather_map(gpu_ctx, oracle_lib, kind):
    from delfem_gb300 import meshgen as mg
    p = {"poisson2d": lambda: mg.poisson2d_square(150, seed=51, coef_sigma=0.5),
         "solid2d": lambda: mg.solid2d_cantilever(200, 80, seed=52, coef_sigma=0.5),
         "poisson3d": lambda: mg.poisson3d_cube(20, seed=53, coef_sigma=1.0),
         "solid3d": lambda: mg.solid3d_cube(12, seed=54, coef_sigma=1.0)}[kind]()
    _check_assembly(gpu_ctx, oracle_lib, p)


def _fan(nfan):
    """A disc of nfan triangles around node 0: node 0 has nfan neighbours and
    nfan element incidences, more than a thread's list holds."""
    from delfem_gb300 import meshgen as mg
    ang = np.linspace(0.0, 2 * np.pi, nfan, endpoint=False)
    coords = np.vstack([[0.0, 0.0], np.column_stack([np.cos(ang), np.sin(ang)])])
    conn = np.array([[0, 1 + i, 1 + (i + 1) % nfan] for i in range(nfan)], dtype=np.int32)
    bc = np.zeros(coords.shape[0], dtype=np.int32)
    bc[1:] = 1
    prm = np.zeros(8)
    prm[0] = 1.0
    prm[1] = 1.0
    coef = np.random.default_rng(5).lognormal(0.0, 0.5, nfan)
    return mg.Problem(mg.POISSON2D, coords, conn, prm, bc, coef=coef, name=f"fan{nfan}")


@pytest.mark.parametrize("nfan", [100, 300])
def test_high_valence_node(gpu_ctx, oracle_lib, nfan):
    """Below and above the per-thread bound (256): the same pattern and
    element assembly either way (above it the host builder takes over).  No
    preconditioner here: a row with 300 dependencies exceeds a sweep step
    record, which the symbolic set-up rejects with DFG_INVALID_ARGUMENT."""
    from delfem_gb300 import linsys as L
    p = _fan(nfan)
    ls = L.LinearSystemField(gpu_ctx, p.nnode, p.b, conn=p.conn)
    try:
        rp, ci = ls.pattern()
        rr, rc = oracle_lib.pattern(p.nnode, p.conn)
        assert np.array_equal(rp, rr) and np.array_equal(ci, rc)
    finally:
        ls.close()
    _check_assembly(gpu_ctx, oracle_lib, p, rr, rc)


def test_pattern_without_some_element_blocks(gpu_ctx, oracle_lib):
    """A pattern given as CRS that lacks some element pairs: those blocks are
    skipped, as CMatDia_BlkCrs::Mearge skips blocks outside the pattern."""
    from delfem_gb300 import meshgen as mg
    p = mg.solid2d_cantilever(30, 12, seed=55, coef_sigma=0.5)
    rp, ci = oracle_lib.pattern(p.nnode, p.conn)
    n = p.nnode
    drop = set()
    rng = np.random.default_rng(6)
    for i in rng.choice(n, 40, replace=False):
        row = ci[rp[i]:rp[i + 1]]
        if row.size:
            j = int(row[rng.integers(row.size)])
            drop.add((int(i), j))
            drop.add((j, int(i)))
    rows = [[int(c) for c in ci[rp[i]:rp[i + 1]] if (i, int(c)) not in drop] for i in range(n)]
    rp2 = np.zeros(n + 1, dtype=np.int32)
    rp2[1:] = np.cumsum([len(r) for r in rows])
    ci2 = np.array([c for r in rows for c in r], dtype=np.int32)
    assert ci2.size < ci.size
    _check_assembly(gpu_ctx, oracle_lib, p, rp2, ci2)


def test_failed_set_mesh_keeps_previous_mesh(gpu_ctx, oracle_lib):
    from delfem_gb300 import capi
    from delfem_gb300 import linsys as L
    from delfem_gb300 import meshgen as mg
    p = mg.poisson2d_square(12, seed=56)
    ls = L.LinearSystemField(gpu_ctx, p.nnode, p.b, conn=p.conn)
    try:
        ls.set_mesh(p.coords, p.conn)
        bad = p.conn.copy()
        bad[3, 1] = p.nnode + 7
        with pytest.raises(capi.DfgError) as e:
            ls.set_mesh(p.coords, bad)
        assert e.value.status == capi.DFG_INVALID_ARGUMENT
        ls.InitializeMarge()
        L.AddLinSys_Poisson(ls, 1.0, 1.0)
        rp, ci = oracle_lib.pattern(p.nnode, p.conn)
        diag, offd, res = oracle_lib.assemble(p, rp, ci)
        gd, go = ls.GetMatrix()
        assert np.array_equal(bits(gd), bits(diag)) and np.array_equal(bits(go), bits(offd))
    finally:
        ls.close()


@pytest.mark.parametrize("dim,kind", [(2, "poisson2d"), (2, "solid2d"), (3, "poisson3d"), (3, "solid3d")])
def test_device_build_on_unstructured_meshes(gpu_ctx, oracle_lib, dim, kind):
    """Delaunay meshes with nodes in random order: irregular valences and
    incidence counts for the device pattern and gather-map build."""
    pytest.importorskip("scipy")
    from delfem_gb300 import meshgen as mg
    co, cn = mg.delaunay_mesh(6000 if dim == 2 else 2500, dim, seed=57 + dim)
    k = {"poisson2d": mg.POISSON2D, "solid2d": mg.SOLID2D, "poisson3d": mg.POISSON3D, "solid3d": mg.SOLID3D}[kind]
    p = mg.mesh_problem(k, co, cn, seed=8, coef_sigma=0.5)
    _check_assembly(gpu_ctx, oracle_lib, p)
