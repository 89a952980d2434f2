"""Generates the golden fixtures in this directory by running the reference
itself (the DelFEM sources compiled headless into oracle/_ref/ref_harness by
``make -C oracle ref``) on small seeded problems.

Each fixture <name>.npz holds the problem (mesh, coefficients, loads,
Dirichlet flags, parameters) and the reference's outputs: the block pattern,
the assembled matrix and right-hand side after FinalizeMarge, the ILU
factor, and the result of LsSol::Solve_PCG (iterations, ratio, solution).
The fixtures in this directory use ILU(0); those in iluk/ use other fill
levels (CPreconditioner_ILU::SetFillInLevel) and add the factor's own block
pattern (ref_rowptr_f, ref_colind_f) and ref_fill_level; those in bicgstab/
hold the result of LsSol::Solve_PBiCGSTAB instead of Solve_PCG (ref_solver);
those in known/ are problems with closed-form answers (known_cases).

Harness problem file (little-endian): int32 magic 0x44464731, kind, nnode,
ndim, nelem, nnoel, b; f64 coords[nnode*ndim]; i32 conn[nelem*nnoel];
i32 has_coef (+ f64 coef[nelem]); f64 params[8]; i32 bcflag[nnode*b];
i32 has_load (+ f64 load[nnode*b]); i32 has_u (+ f64 u); i32 has_v (+ f64 v);
f64 tol; i32 maxit.  The result file layout is read by meshgen.read_result.

Run from the repository root:  python tests/golden/make_golden.py [ilu0|iluk|bicgstab|known|all]
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from delfem_gb300 import meshgen as mg  # noqa: E402
import oracle as O  # noqa: E402


def cases():
    return [
        mg.poisson2d_square(8, seed=11),
        mg.poisson2d_square(12, seed=12, coef_sigma=0.5),
        mg.solid2d_cantilever(10, 5, seed=13, coef_sigma=0.5),
        mg.solid2d_cantilever(6, 3, seed=14, coef_sigma=0.0),
        mg.solid3d_cube(3, seed=15, coef_sigma=1.0),
        mg.solid3d_cube(4, seed=16, coef_sigma=0.0, jitter=0.15),
        mg.poisson3d_cube(4, seed=17),
        mg.poisson3d_cube(5, seed=18, coef_sigma=1.0),
        mg.diffusion2d_square(6, seed=19),
    ]


def iluk_cases():
    """(problem, fill level): the solid default ILU(1) of CEqnSystem_Solid2D
    (eqnsys_solid.cpp:640), higher levels, a level whose pattern is smaller
    than the level below it, and the unlimited level -1 (complete LU)."""
    return [
        (mg.solid2d_cantilever(10, 5, seed=13, coef_sigma=0.5), 1),
        (mg.poisson2d_square(12, seed=12, coef_sigma=0.5), 2),
        (mg.poisson2d_square(8, seed=11), 3),
        (mg.solid3d_cube(3, seed=15, coef_sigma=1.0), 1),
        (mg.poisson3d_cube(5, seed=18, coef_sigma=1.0), 2),
        (mg.solid2d_cantilever(6, 3, seed=14, coef_sigma=0.0), -1),
        (mg.diffusion2d_square(6, seed=19), 1),
    ]


def bicgstab_cases():
    """(problem, fill level): Solve_PBiCGSTAB on ILU(0) and ILU(1), an
    iteration limit that stops it early (the reference then returns true with
    the ratio untouched) and a zero right-hand side (immediate return)."""
    zero = mg.poisson2d_square(6, seed=23)
    zero.params = zero.params.copy()
    zero.params[1] = 0.0
    zero.load = None
    zero.name = "poisson2d_6x6_zero"
    short = mg.solid2d_cantilever(10, 5, seed=24, coef_sigma=0.5)
    short.maxit = 5
    short.name = "solid2d_10x5_maxit5"
    return [
        (mg.poisson2d_square(12, seed=12, coef_sigma=0.5), 0),
        (mg.solid2d_cantilever(10, 5, seed=13, coef_sigma=0.5), 0),
        (mg.solid2d_cantilever(10, 5, seed=13, coef_sigma=0.5), 1),
        (mg.solid3d_cube(3, seed=15, coef_sigma=1.0), 0),
        (mg.poisson3d_cube(5, seed=18, coef_sigma=1.0), 1),
        (mg.diffusion2d_square(6, seed=19), 0),
        (short, 0),
        (zero, 0),
    ]


def known_cases():
    """Problems whose answers are known in closed form; the reference's own
    run of each is committed beside it.
    * A 2 x 2 Poisson grid without jitter, all sides fixed: its one free node
      has the stencil 4 / -1 (axis neighbours) / 0 (along the split diagonal),
      right-hand side source * h^2 = 0.25 and solution 0.0625.
    * Linear fields, which P1 elements reproduce exactly, on jittered meshes
      with uniform material and no source or body force.  The field is set on
      the boundary (Dirichlet lifting: the field value enters the residual as
      -K u), and field + update must equal it everywhere.  Cases: 2D Poisson,
      2D elasticity (both displacement components) and 3D Poisson."""
    out = []
    coords, conn = mg.tri_grid(2, 2)
    bc = np.ones(coords.shape[0], dtype=np.int32)
    bc[4] = 0  # the centre node
    prm = np.zeros(8); prm[0] = 1.0; prm[1] = 1.0
    out.append(mg.Problem(mg.POISSON2D, coords, conn, prm, bc, tol=1e-12, name="poisson2d_2x2"))

    def boundary_flags(conn, nnode, b):
        f = np.zeros(nnode, dtype=np.int32)
        f[mg.boundary_nodes(conn)] = 1
        return np.repeat(f, b).astype(np.int32)

    rng = np.random.default_rng(31)
    coords, conn = mg.tri_grid(6, 5, 1.0, 1.0, 0.2, rng)
    bc = boundary_flags(conn, coords.shape[0], 1)
    g = 0.7 + 1.3 * coords[:, 0] - 0.4 * coords[:, 1]
    prm = np.zeros(8); prm[0] = 1.0
    out.append(mg.Problem(mg.POISSON2D, coords, conn, prm, bc, u=g * bc, tol=1e-12, name="poisson2d_linear"))

    coords, conn = mg.tri_grid(7, 4, 2.0, 1.0, 0.2, rng)
    bc = boundary_flags(conn, coords.shape[0], 2)
    x, y = coords[:, 0], coords[:, 1]
    g = np.stack([0.01 + 0.02 * x - 0.03 * y, -0.02 + 0.015 * x + 0.01 * y], axis=1).ravel()
    E, nu = 1.0, 0.3
    prm = np.zeros(8); prm[0] = E * nu / ((1 + nu) * (1 - 2 * nu)); prm[1] = E / (2 * (1 + nu))
    out.append(mg.Problem(mg.SOLID2D, coords, conn, prm, bc, u=g * bc, tol=1e-12, name="solid2d_linear"))

    coords, conn = mg.tet_grid(3, 3, 3, jitter=0.15, rng=rng)
    bc = boundary_flags(conn, coords.shape[0], 1)
    g = 0.5 + coords[:, 0] - 2.0 * coords[:, 1] + 0.25 * coords[:, 2]
    prm = np.zeros(8); prm[0] = 1.0
    out.append(mg.Problem(mg.POISSON3D, coords, conn, prm, bc, u=g * bc, tol=1e-12, name="poisson3d_linear"))
    return out


def fixture_name(p: mg.Problem, k: int, fill_level: int = 0) -> str:
    tag = "coef" if p.coef is not None else "uniform"
    lev = "" if fill_level == 0 else (f"_ilu{fill_level}" if fill_level > 0 else "_ilufull")
    return f"{k:02d}_{p.name.replace('^', 'c')}_{tag}{lev}"


def write_fixture(path: str, p: mg.Problem, fill_level: int, solver: str = "pcg") -> None:
    R = O.run_reference_harness(p, fill_level, solver)
    d = dict(kind=p.kind, coords=p.coords, conn=p.conn, params=p.params, bcflag=p.bcflag, tol=p.tol,
             maxit=p.maxit)
    for nm in ("coef", "load", "u", "v"):
        a = getattr(p, nm)
        if a is not None:
            d[nm] = a
    for nm in ("rowptr", "colind", "diag", "offd", "rhs", "fdiag", "foffd", "x"):
        d["ref_" + nm] = R[nm]
    for nm in ("norm_res", "ilu_ok", "converged", "iter", "conv"):
        d["ref_" + nm] = np.array(R[nm])
    if solver != "pcg":
        d["ref_solver"] = np.array(solver)
    if fill_level != 0 or solver != "pcg":
        d["ref_fill_level"] = np.array(fill_level)
        d["ref_rowptr_f"] = R["rowptr_f"]
        d["ref_colind_f"] = R["colind_f"]
    np.savez_compressed(path, **d)
    print(f"{path}: n={R['n']} b={R['b']} nnz={R['nnz']} nnz_f={R['colind_f'].size} iter={R['iter']} "
          f"conv={R['conv']:.3e}")


def main():
    if not O.harness_available():
        raise SystemExit("oracle/_ref/ref_harness is missing: run `make -C oracle ref` where the reference exists")
    which = sys.argv[1] if len(sys.argv) > 1 else "all"
    here = os.path.dirname(os.path.abspath(__file__))
    if which in ("ilu0", "all"):
        for k, p in enumerate(cases()):
            write_fixture(os.path.join(here, fixture_name(p, k) + ".npz"), p, 0)
    if which in ("iluk", "all"):
        os.makedirs(os.path.join(here, "iluk"), exist_ok=True)
        for k, (p, lev) in enumerate(iluk_cases()):
            write_fixture(os.path.join(here, "iluk", fixture_name(p, k, lev) + ".npz"), p, lev)
    if which in ("known", "all"):
        os.makedirs(os.path.join(here, "known"), exist_ok=True)
        for k, p in enumerate(known_cases()):
            write_fixture(os.path.join(here, "known", fixture_name(p, k) + ".npz"), p, 0)
    if which in ("bicgstab", "all"):
        os.makedirs(os.path.join(here, "bicgstab"), exist_ok=True)
        for k, (p, lev) in enumerate(bicgstab_cases()):
            write_fixture(os.path.join(here, "bicgstab", fixture_name(p, k, lev) + ".npz"), p, lev, "bicgstab")


if __name__ == "__main__":
    main()
