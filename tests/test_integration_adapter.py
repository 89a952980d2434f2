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


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "include", "delfem")), reason="reference headers absent")
def test_adapter_compiles_and_links(tmp_path):
    from delfem_gb300 import build as B
    lib = B.build()
    subprocess.run(["make", "-s", "-j8", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    exe = str(tmp_path / "integration")
    cmd = ["g++", "-O1", "-std=c++17", "-w", "-include", "cassert", f"-I{REF}/include", f"-I{ROOT}/include",
           os.path.join(ROOT, "tests", "cpu", "integration_main.cpp"),
           os.path.join(ROOT, "oracle", "_ref", "libdfm_ref.a"), lib, f"-Wl,-rpath,{os.path.dirname(lib)}",
           "-o", exe]
    subprocess.run(cmd, check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
