"""Shared test helpers.  Tests marked ``gpu`` need a CUDA device and libdfg
built for sm_103a; everything else runs on the CPU."""
from __future__ import annotations

import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and libdfg")


def golden_files():
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


def golden_iluk_files():
    """Fixtures with an ILU fill level other than 0 (ref_fill_level)."""
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, "iluk", "*.npz")))


def golden_bicgstab_files():
    """Fixtures solved by Solve_PBiCGSTAB (ref_solver), ILU(ref_fill_level)."""
    return sorted(glob.glob(os.path.join(GOLDEN_DIR, "bicgstab", "*.npz")))


def load_golden(path):
    """Returns (problem, reference outputs) of one committed fixture."""
    from delfem_gb300 import meshgen as mg
    z = np.load(path)
    p = mg.Problem(kind=int(z["kind"]), coords=z["coords"], conn=z["conn"], params=z["params"],
                   bcflag=z["bcflag"], coef=z["coef"] if "coef" in z else None,
                   load=z["load"] if "load" in z else None, u=z["u"] if "u" in z else None,
                   v=z["v"] if "v" in z else None, tol=float(z["tol"]), maxit=int(z["maxit"]),
                   name=os.path.basename(path)[:-4])
    ref = {k[4:]: z[k] for k in z.files if k.startswith("ref_")}
    return p, ref


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_ctx():
    from delfem_gb300 import build as B
    B.build()
    from delfem_gb300 import linsys
    ctx = linsys.Context(0)
    yield ctx
    ctx.close()
