"""Whole-path driver for a ``meshgen.Problem``: pattern, mesh upload,
Dirichlet flags, symbolic ILU set-up (fill level 0 unless asked), then per
solve InitializeMarge -> AddLinSys_* -> extra loads -> FinalizeMarge -> ILU
numeric -> PCG.

This is the sequence of the reference's low-level drivers
(test_glut_lowlev/solid2d/main.cpp:186-298) expressed through the drop-in
interface in ``linsys``.
"""
from __future__ import annotations

import time

import numpy as np

from . import linsys as L
from . import meshgen as mg


class FESolve:
    def __init__(self, ctx: L.Context, p: mg.Problem, fill_level: int = 0, sweep_mode: int = 0):
        self.ctx, self.p = ctx, p
        self.ls = L.LinearSystemField(ctx, p.nnode, p.b, conn=p.conn)
        self.ls.set_mesh(p.coords, p.conn)
        if p.coef is not None:
            self.ls.set_coef(p.coef)
        if p.u is not None or p.v is not None:
            self.ls.set_field(p.u, p.v)
        self.ls.SetFixedBoundaryCondition(p.bcflag)
        if p.load is not None:
            self.ls.SetLoad(p.load)
        self.prec = L.PreconditionerILU(ctx)
        self.prec.SetFillInLevel(fill_level)
        if sweep_mode:
            self.prec.SetSweepMode(sweep_mode)
        self.prec.SetLinearSystem(self.ls)

    def assemble(self) -> float:
        p, ls = self.p, self.ls
        P = [float(x) for x in p.params]
        ls.InitializeMarge()
        if p.kind in (mg.POISSON2D, mg.POISSON3D):
            L.AddLinSys_Poisson(ls, P[0], P[1])
        elif p.kind == mg.DIFFUSION2D:
            L.AddLinSys_Diffusion(P[4], P[3], ls, P[0], P[1], P[2])
        elif p.kind == mg.SOLID2D:
            L.AddLinSys_LinearSolid2D_Static(ls, P[0], P[1], P[2], P[3], P[4])
        elif p.kind == mg.SOLID3D:
            L.AddLinSys_LinearSolid3D_Static(ls, P[0], P[1], P[2], P[3], P[4], P[5])
        return ls.FinalizeMarge()  # adds the resident load, then the Dirichlet rows

    def factor(self) -> bool:
        return self.prec.SetValue(self.ls)

    def solve(self, mode: str = "fp64", tol: float | None = None, maxit: int | None = None,
              target_true: bool = False, solver: str = "pcg") -> dict:
        """mode: "fp64" (LsSol::Solve_PCG semantics unless target_true), "mixed"
        (FP32 factor/sweeps/SpMV/vectors + FP64 refinement, always on the true
        residual) or "fp32f" (FP32 factor and sweeps only).  solver "bicgstab"
        runs LsSol::Solve_PBiCGSTAB instead (mode fp64 only; its stop test is
        the recursive residual, target_true does not apply)."""
        tol = self.p.tol if tol is None else tol
        maxit = self.p.maxit if maxit is None else maxit
        if solver == "bicgstab":
            ok, conv, it = L.Solve_PBiCGSTAB(tol, maxit, self.ls, self.prec, mode)
            return dict(converged=ok, conv=conv, iter=it, refinements=0)
        if mode == "fp64" and not target_true:
            ok, conv, it = L.Solve_PCG(tol, maxit, self.ls, self.prec)
            return dict(converged=ok, conv=conv, iter=it, refinements=0)
        if mode == "mixed":
            ok, conv, it, outer = L.Solve_PCG_Mixed(tol, maxit, self.ls, self.prec)
            return dict(converged=ok, conv=conv, iter=it, refinements=outer)
        ok, conv, it, refin = L.Solve_PCG_ex(tol, maxit, self.ls, self.prec, mode, target_true)
        return dict(converged=ok, conv=conv, iter=it, refinements=refin)

    def run(self, mode: str = "fp64", tol: float | None = None, maxit: int | None = None,
            target_true: bool = False, solver: str = "pcg") -> dict:
        t0 = time.perf_counter()
        norm_res = self.assemble()
        self.ctx.synchronize()
        t1 = time.perf_counter()
        ok = self.factor()
        self.ctx.synchronize()
        t2 = time.perf_counter()
        out = self.solve(mode, tol, maxit, target_true, solver)
        t3 = time.perf_counter()
        out.update(norm_res=norm_res, ilu_ok=ok, t_assemble=t1 - t0, t_ilu=t2 - t1, t_solve=t3 - t2)
        return out

    def solution(self) -> np.ndarray:
        return self.ls.GetUpdate()

    def close(self):
        self.prec.close()
        self.ls.close()
