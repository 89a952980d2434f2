"""include/dfg_delfem.hpp compiles against the reference's own headers and
links with the reference library and libdfg (the reference-side binding a
DelFEM maintainer would add); without a GPU the program stops after
creating the context.  Needs the reference sources, so it runs only where
they are present."""
import os
import subprocess

import pytest

from conftest import ROOT
from oracle import reference_dir

REF = reference_dir()


needs_ref = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include", "delfem")),
                               reason="reference headers absent (set DFG_REFERENCE_DIR)")


def _build_program(tmp_path):
    """The reference library (oracle/Makefile `ref`, from the reference's own
    sources at REF) and tests/cpu/integration_main.cpp linked against it and
    libdfg."""
    from delfem_gb300 import build as B
    lib = B.build()
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    exe = str(tmp_path / "integration")
    cmd = ["g++", "-O1", "-std=c++17", "-w", "-include", "cassert", f"-I{REF}/include", f"-I{ROOT}/include",
           os.path.join(ROOT, "tests", "cpu", "integration_main.cpp"),
           os.path.join(ROOT, "oracle", "_ref", "libdfm_ref.a"), lib, f"-Wl,-rpath,{os.path.dirname(lib)}",
           "-o", exe]
    subprocess.run(cmd, check=True)
    return exe


@needs_ref
def test_adapter_compiles_and_links(tmp_path):
    exe = _build_program(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr


@needs_ref
@pytest.mark.gpu
def test_adapter_drives_the_gpu(tmp_path):
    """On a GPU: the reference's own LsSol::Solve_PCG and Solve_PBiCGSTAB over
    CLinearSystem_FieldGPU, CPreconditioner_ILU_GPU inside the reference's
    host CLinearSystem_Field beside its CPreconditioner_ILU, and CMatSolverGPU
    beside MatVec::Sol::Solve_PCG: every pair converges with iterations
    within 2 and solutions within 1e-6 relative L2 (the program's exit code
    says which check failed)."""
    exe = _build_program(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    for line in ("host system, reference Solve_PCG", "reference loop:", "BiCGSTAB reference loop",
                 "matrix-level PCG reference"):
        assert line in r.stdout, r.stdout
