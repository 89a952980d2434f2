"""GiD mesh input (dfg_mesh_read_gid, a host entry point of libdfg: no device
needed).  Parity: the reference's own readers (Msh::CMesher2D / Msh::CMesh3D
::ReadFromFile_GiDMsh, run through oracle/_ref/ref_harness) on the
reference's input meshes give bit-identical nodes and elements, and a whole
solve on such a mesh matches the reference's; these read the reference's
files and run only where its sources are present.  Round trips through the
writer and the error cases run everywhere."""
import os
import struct

import numpy as np
import pytest

from conftest import bits
from oracle import reference_dir

REF_MESHES = os.path.join(reference_dir(), "test_glut", "input_file")
TRI = ["rect_tri", "rect_tri2", "rect_tri3", "hexa_tri"]
TET = ["cylinder_tet", "cylinder_tet2", "redtsolid_tet"]


def _lib_built():
    from delfem_gb300 import build as B
    B.build()


def _ref_dump(kind, path, tmp_path):
    import oracle as O
    out = str(tmp_path / "mesh.bin")
    import subprocess
    subprocess.run([O.HARNESS, kind, path, out], check=True, stdout=subprocess.DEVNULL)
    raw = open(out, "rb").read()
    magic, ndim, nnoel, nnode, nelem = struct.unpack_from("<5i", raw, 0)
    assert magic == 0x44464D31
    co = np.frombuffer(raw, "<f8", nnode * ndim, 20).reshape(nnode, ndim)
    cn = np.frombuffer(raw, "<i4", nelem * nnoel, 20 + 8 * nnode * ndim).reshape(nelem, nnoel)
    return co, cn


needs_ref = pytest.mark.skipif(not os.path.isdir(REF_MESHES), reason="reference input meshes absent")


@needs_ref
@pytest.mark.parametrize("name", TRI + TET)
def test_reader_matches_reference_reader(name, tmp_path, oracle_lib):
    from delfem_gb300 import meshgen as mg
    import oracle as O
    _lib_built()
    if not O.harness_available():
        pytest.skip("reference harness not built")
    path = os.path.join(REF_MESHES, name + ".msh")
    co, cn = mg.read_gid_msh(path)
    rco, rcn = _ref_dump("--mesh2d" if name in TRI else "--mesh3d", path, tmp_path)
    assert co.shape == rco.shape and cn.shape == rcn.shape
    assert np.array_equal(bits(co), bits(rco))
    assert np.array_equal(cn, rcn)


@needs_ref
@pytest.mark.parametrize("name,kind", [("rect_tri", "solid2d"), ("hexa_tri", "poisson2d"),
                                       ("cylinder_tet", "poisson3d")])
def test_solve_on_reference_mesh_matches_reference(name, kind, oracle_lib):
    """The oracle's whole path on a mesh read by the library equals the
    reference's own run on it, bit for bit."""
    from delfem_gb300 import meshgen as mg
    import oracle as O
    _lib_built()
    if not O.harness_available():
        pytest.skip("reference harness not built")
    co, cn = mg.read_gid_msh(os.path.join(REF_MESHES, name + ".msh"))
    k = {"solid2d": mg.SOLID2D, "poisson2d": mg.POISSON2D, "poisson3d": mg.POISSON3D}[kind]
    p = mg.mesh_problem(k, co, cn, seed=3, coef_sigma=0.5, name=name)
    R = O.run_reference_harness(p)
    out = oracle_lib.solve(p)
    assert R["converged"] and out["converged"]
    for key in ("diag", "offd", "rhs", "fdiag", "foffd", "x"):
        assert np.array_equal(bits(out[key]), bits(R[key])), key
    assert out["iter"] == R["iter"]


@pytest.mark.parametrize("dim", [2, 3])
def test_write_read_round_trip(dim, tmp_path):
    from delfem_gb300 import meshgen as mg
    _lib_built()
    rng = np.random.default_rng(dim)
    if dim == 2:
        co, cn = mg.tri_grid(7, 5, 1.4, 1.0, 0.2, rng)
    else:
        co, cn = mg.tet_grid(3, 4, 2, jitter=0.15, rng=rng)
    path = str(tmp_path / "m.msh")
    mg.write_gid_msh(path, co, cn)
    rco, rcn = mg.read_gid_msh(path)
    assert np.array_equal(bits(rco), bits(np.asarray(co, dtype=np.float64)))
    assert np.array_equal(rcn, cn)


def test_planar_triangles_in_another_plane(tmp_path):
    """Triangles in the y-z plane: x is dropped and (y, z) kept, the order the
    reference's 2D reader uses for that plane."""
    from delfem_gb300 import meshgen as mg
    _lib_built()
    co, cn = mg.tri_grid(4, 3, 1.0, 1.0, 0.1, np.random.default_rng(5))
    co3 = np.column_stack([np.full(len(co), 2.5), co[:, 0], co[:, 1]])
    path = str(tmp_path / "yz.msh")
    with open(path, "w") as f:
        f.write("MESH    dimension 3 ElemType Triangle  Nnode 3\nCoordinates\n")
        for i, c in enumerate(co3):
            f.write(f"{i + 1} {c[0]:.17g} {c[1]:.17g} {c[2]:.17g}\n")
        f.write("end coordinates\n\nElements\n")
        for e, v in enumerate(cn):
            f.write(f"{e + 1} {v[0] + 1} {v[1] + 1} {v[2] + 1}\n")
        f.write("end elements\n")
    rco, rcn = mg.read_gid_msh(path)
    assert np.array_equal(bits(rco), bits(co3[:, 1:])) and np.array_equal(rcn, cn)


@pytest.mark.parametrize("text,why", [
    ("MESH dimension 3 ElemType Quadrilateral Nnode 4\nCoordinates\nend coordinates\n", "element type"),
    ("MESH dimension 3 ElemType Triangle Nnode 3\nCoordinates\n1 0 0 0\n3 1 0 0\nend coordinates\n", "node ids"),
    ("MESH dimension 3 ElemType Triangle Nnode 3\nCoordinates\n1 0 0 0\n2 1 0 0\n3 0 1 1\n4 1 1 0\n"
     "end coordinates\n\nElements\n1 1 2 3\n2 2 4 3\nend elements\n", "not planar"),
    ("MESH dimension 3 ElemType Tetrahedra Nnode 4\nCoordinates\n1 0 0 0\n2 1 0 0\n3 0 1 0\n4 0 0 1\n"
     "end coordinates\n\nElements\n1 1 2 3 9\nend elements\n", "out of range"),
    ("hello\n", "header"),
])
def test_reader_rejects_malformed_files(text, why, tmp_path):
    from delfem_gb300 import capi
    from delfem_gb300 import meshgen as mg
    _lib_built()
    path = str(tmp_path / "bad.msh")
    open(path, "w").write(text)
    with pytest.raises(capi.DfgError) as e:
        mg.read_gid_msh(path)
    assert e.value.status == capi.DFG_INVALID_ARGUMENT and why in str(e.value)


def test_reader_missing_file():
    from delfem_gb300 import capi
    from delfem_gb300 import meshgen as mg
    _lib_built()
    with pytest.raises(capi.DfgError):
        mg.read_gid_msh("/nonexistent/mesh.msh")


def test_boundary_nodes_of_grids():
    from delfem_gb300 import meshgen as mg
    co, cn = mg.tri_grid(5, 4, 1.0, 1.0, 0.0, np.random.default_rng(1))
    b = mg.boundary_nodes(cn)
    x, y = co[:, 0], co[:, 1]
    on = np.nonzero((x == 0) | (x == 1) | (y == 0) | (y == 1))[0]
    assert np.array_equal(b, on)
    co, cn = mg.tet_grid(3, 3, 3)
    b = mg.boundary_nodes(cn)
    on = np.nonzero(((co == 0) | (co == 1)).any(axis=1))[0]
    assert np.array_equal(b, on)
