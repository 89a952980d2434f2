"""Host-side mirror of DelFEM's linear-system / preconditioner / solver
interface over libdfg's C ABI.

Names and argument meanings follow the reference so call sites read like
its own drivers (test_glut_lowlev/solid2d/main.cpp:186-298):

    ls = LinearSystemField(ctx, nblk, blklen, conn=...)   # AddPattern_Field
    ls.set_mesh(coords, conn); ls.SetFixedBoundaryCondition(flags)
    prec = PreconditionerILU(ctx); prec.SetFillInLevel(0); prec.SetLinearSystem(ls)
    ls.InitializeMarge(); AddLinSys_Poisson(ls, alpha, source); ls.FinalizeMarge()
    prec.SetValue(ls)
    ok, conv, it = Solve_PCG(1e-8, 1000, ls, prec)

Vector slots: -1 residual, -2 update, >= 0 work vectors
(include/delfem/ls/linearsystem_interface_solver.h:39-82).
"""
from __future__ import annotations

import ctypes
import weakref

import numpy as np

from . import capi
from .capi import check, lib


def _p(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


class Context:
    """One CUDA device + stream (dfg_ctx).  Systems, preconditioners and
    servers made on it register here; closing the context closes those still
    open first (the C ABI wants them destroyed before their context)."""

    def __init__(self, device: int = 0):
        self._children = weakref.WeakSet()
        h = ctypes.c_void_p()
        st = lib().dfg_ctx_create(device, ctypes.byref(h))
        if st != capi.DFG_OK:
            raise capi.DfgError(st, "dfg_ctx_create", lib().dfg_last_error(None).decode(errors="replace"))
        self.h = h

    def adopt(self, obj) -> None:
        """Registers an object with a native handle on this context; it must
        have close() and a _close_order (lower closes first)."""
        self._children.add(obj)

    def synchronize(self):
        check(self.h, lib().dfg_ctx_synchronize(self.h), "dfg_ctx_synchronize")

    @property
    def stream(self) -> int:
        h = ctypes.c_void_p()
        check(self.h, lib().dfg_ctx_get_stream(self.h, ctypes.byref(h)), "dfg_ctx_get_stream")
        return int(h.value or 0)

    @property
    def kernel_launches(self) -> int:
        return int(lib().dfg_ctx_kernel_launches(self.h))

    def last_error(self) -> str:
        return lib().dfg_last_error(self.h).decode()

    def close(self):
        if self.h:
            for c in sorted(list(self._children), key=lambda o: o._close_order):
                c.close()
            lib().dfg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LinearSystemField:
    """Fem::Ls::CLinearSystem_Field (include/delfem/femls/linearsystem_field.h:67-172)
    restricted to one field segment of square blocks."""

    def __init__(self, ctx: Context, nblk: int, blklen: int, conn=None, rowptr=None, colind=None):
        self.ctx = ctx
        self.n, self.b = int(nblk), int(blklen)
        h = ctypes.c_void_p()
        if conn is not None:
            conn = _i32(conn)
            st = lib().dfg_system_create_from_elements(ctx.h, self.n, self.b, conn.shape[0], conn.shape[1], _p(conn),
                                                       ctypes.byref(h))
        else:
            rowptr, colind = _i32(rowptr), _i32(colind)
            st = lib().dfg_system_create(ctx.h, self.n, self.b, _p(rowptr), _p(colind), ctypes.byref(h))
        check(ctx.h, st, "dfg_system_create")
        self.h = h
        ctx.adopt(self)
        nnz = ctypes.c_longlong()
        lib().dfg_system_info(self.h, None, None, ctypes.byref(nnz))
        self.nnz = int(nnz.value)

    # -- pattern / mesh ------------------------------------------------------
    def pattern(self):
        rowptr = np.zeros(self.n + 1, dtype=np.int32)
        colind = np.zeros(max(self.nnz, 1), dtype=np.int32)
        lib().dfg_system_get_pattern(self.h, _p(rowptr), _p(colind))
        return rowptr, colind[: self.nnz]

    def set_mesh(self, coords, conn):
        coords, conn = _f64(coords), _i32(conn)
        check(self.ctx.h, lib().dfg_system_set_mesh(self.h, coords.shape[1], _p(coords), conn.shape[0],
                                                    conn.shape[1], _p(conn)), "dfg_system_set_mesh")

    def set_coef(self, coef):
        c = None if coef is None else _f64(coef)
        check(self.ctx.h, lib().dfg_system_set_coef(self.h, _p(c)), "dfg_system_set_coef")

    def set_field(self, u=None, v=None):
        u = None if u is None else _f64(u)
        v = None if v is None else _f64(v)
        check(self.ctx.h, lib().dfg_system_set_field(self.h, _p(u), _p(v)), "dfg_system_set_field")

    def UpdateValueOfField(self, fdt: int = 0):
        """CLinearSystem_Field::UpdateValueOfField on the resident field:
        value (fdt 0) or velocity (fdt 1) += update, on the device."""
        check(self.ctx.h, lib().dfg_system_update_field(self.h, fdt), "dfg_system_update_field")

    def get_field(self):
        """Host copies (u, v) of the resident field."""
        u = np.zeros(self.n * self.b)
        v = np.zeros(self.n * self.b)
        check(self.ctx.h, lib().dfg_system_get_field(self.h, _p(u), _p(v)), "dfg_system_get_field")
        return u, v

    def SetLoad(self, f):
        """Resident nodal load added at every FinalizeMarge (None clears it)."""
        ff = None if f is None else _f64(f)
        check(self.ctx.h, lib().dfg_system_set_load(self.h, _p(ff)), "dfg_system_set_load")

    def SetFixedBoundaryCondition(self, flags):
        f = _i32(flags)
        check(self.ctx.h, lib().dfg_set_bcflags(self.h, _p(f)), "dfg_set_bcflags")

    # -- assembly --------------------------------------------------------------
    def InitializeMarge(self):
        check(self.ctx.h, lib().dfg_initialize_marge(self.h), "dfg_initialize_marge")

    def AddResidual(self, f):
        f = _f64(f)
        check(self.ctx.h, lib().dfg_add_residual(self.h, _p(f)), "dfg_add_residual")

    def FinalizeMarge(self) -> float:
        r = ctypes.c_double()
        check(self.ctx.h, lib().dfg_finalize_marge(self.h, ctypes.byref(r)), "dfg_finalize_marge")
        return r.value

    def GetMatrix(self):
        bs = self.b * self.b
        diag = np.zeros(self.n * bs)
        offd = np.zeros(max(self.nnz, 1) * bs)
        check(self.ctx.h, lib().dfg_get_matrix(self.h, _p(diag), _p(offd)), "dfg_get_matrix")
        return diag, offd[: self.nnz * bs]

    def SetMatrix(self, diag, offd):
        diag, offd = _f64(diag), _f64(offd)
        check(self.ctx.h, lib().dfg_set_matrix(self.h, _p(diag), _p(offd)), "dfg_set_matrix")

    def GetVector(self, iv: int) -> np.ndarray:
        out = np.zeros(self.n * self.b)
        check(self.ctx.h, lib().dfg_get_vector(self.h, iv, _p(out)), "dfg_get_vector")
        return out

    def SetVector(self, iv: int, v):
        v = _f64(v)
        check(self.ctx.h, lib().dfg_set_vector(self.h, iv, _p(v)), "dfg_set_vector")

    def GetResidual(self):
        return self.GetVector(-1)

    def GetUpdate(self):
        return self.GetVector(-2)

    # -- LsSol::ILinearSystem_Sol virtuals --------------------------------------
    def GetTmpVectorArySize(self) -> int:
        n = ctypes.c_uint()
        check(self.ctx.h, lib().dfg_get_tmp_vector_size(self.h, ctypes.byref(n)), "dfg_get_tmp_vector_size")
        return n.value

    def ReSizeTmpVecSolver(self, size: int) -> bool:
        check(self.ctx.h, lib().dfg_resize_tmp_vec(self.h, size), "dfg_resize_tmp_vec")
        return True

    def DOT(self, iv1: int, iv2: int) -> float:
        r = ctypes.c_double()
        check(self.ctx.h, lib().dfg_dot(self.h, iv1, iv2, ctypes.byref(r)), "dfg_dot")
        return r.value

    def COPY(self, iv1: int, iv2: int) -> bool:
        check(self.ctx.h, lib().dfg_copy(self.h, iv1, iv2), "dfg_copy")
        return True

    def SCAL(self, alpha: float, iv1: int) -> bool:
        check(self.ctx.h, lib().dfg_scal(self.h, alpha, iv1), "dfg_scal")
        return True

    def AXPY(self, alpha: float, iv1: int, iv2: int) -> bool:
        check(self.ctx.h, lib().dfg_axpy(self.h, alpha, iv1, iv2), "dfg_axpy")
        return True

    def MATVEC(self, alpha: float, iv1: int, beta: float, iv2: int) -> bool:
        check(self.ctx.h, lib().dfg_matvec(self.h, alpha, iv1, beta, iv2), "dfg_matvec")
        return True

    def true_residual(self, b=None) -> float:
        r = ctypes.c_double()
        bb = None if b is None else _f64(b)
        check(self.ctx.h, lib().dfg_true_residual(self.h, _p(bb), ctypes.byref(r)), "dfg_true_residual")
        return r.value

    _close_order = 2

    def close(self):
        if getattr(self, "h", None):
            if self.ctx.h:  # after its context the handle is only dropped
                lib().dfg_system_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PreconditionerILU:
    """LsSol::CPreconditioner_ILU (include/delfem/ls/preconditioner.h:59-108):
    ILU(0) by default; SetFillInLevel(k) before SetLinearSystem gives the
    reference's level-of-fill ILU(k) (-1: no level limit)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        h = ctypes.c_void_p()
        check(ctx.h, lib().dfg_precond_create(ctx.h, ctypes.byref(h)), "dfg_precond_create")
        self.h = h
        ctx.adopt(self)
        self.ls = None

    def SetFillInLevel(self, lev: int):
        check(self.ctx.h, lib().dfg_precond_set_fill_level(self.h, lev), "dfg_precond_set_fill_level")

    def SetSweepMode(self, mode: int):
        """0: timed choice (default), 1: ranged, 2: level-scheduled, 3: one-CTA sweeps."""
        check(self.ctx.h, lib().dfg_precond_set_sweep_mode(self.h, mode), "dfg_precond_set_sweep_mode")

    def GetSweepMode(self):
        """(forward, backward) kinds chosen at the symbolic set-up: 1 ranged, 2 level-scheduled."""
        f, b = ctypes.c_int(), ctypes.c_int()
        check(self.ctx.h, lib().dfg_precond_get_sweep_mode(self.h, ctypes.byref(f), ctypes.byref(b)),
              "dfg_precond_get_sweep_mode")
        return f.value, b.value

    def GetSweepTiming(self):
        """Set-up timings (ms per FP32 sweep) behind the schedule choice:
        forward ranged, forward level-scheduled, backward ranged, backward
        level-scheduled (-1: not timed)."""
        ms = np.zeros(4, dtype=np.float32)
        check(self.ctx.h, lib().dfg_precond_get_sweep_timing(self.h, _p(ms)), "dfg_precond_get_sweep_timing")
        return [float(x) for x in ms]

    def GetSoloTiming(self):
        """Set-up timings (ms per FP32 sweep) of the one-CTA kind: forward,
        backward (-1: not timed)."""
        ms = np.zeros(2, dtype=np.float32)
        check(self.ctx.h, lib().dfg_precond_get_solo_timing(self.h, _p(ms)), "dfg_precond_get_solo_timing")
        return [float(x) for x in ms]

    def SetLinearSystem(self, ls: LinearSystemField):
        check(self.ctx.h, lib().dfg_precond_set_linear_system(self.h, ls.h), "dfg_precond_set_linear_system")
        self.ls = ls

    def SetValue(self, ls: LinearSystemField) -> bool:
        st = lib().dfg_precond_set_value(self.h, ls.h)
        if st == capi.DFG_SINGULAR_PIVOT:
            return False
        check(self.ctx.h, st, "dfg_precond_set_value")
        return True

    def SolvePrecond(self, ls: LinearSystemField, iv: int) -> bool:
        check(self.ctx.h, lib().dfg_precond_solve(self.h, ls.h, iv), "dfg_precond_solve")
        return True

    def GetPattern(self):
        """(rowptr, colind) of the factor: A's pattern plus fill-in."""
        nnz = ctypes.c_longlong()
        check(self.ctx.h, lib().dfg_precond_get_pattern(self.h, ctypes.byref(nnz), None, None),
              "dfg_precond_get_pattern")
        rowptr = np.zeros(self.ls.n + 1, dtype=np.int32)
        colind = np.zeros(max(nnz.value, 1), dtype=np.int32)
        check(self.ctx.h, lib().dfg_precond_get_pattern(self.h, None, _p(rowptr), _p(colind)),
              "dfg_precond_get_pattern")
        return rowptr, colind[: nnz.value]

    def GetFactor(self):
        ls = self.ls
        bs = ls.b * ls.b
        nnz = ctypes.c_longlong()
        check(self.ctx.h, lib().dfg_precond_get_pattern(self.h, ctypes.byref(nnz), None, None),
              "dfg_precond_get_pattern")
        fdiag = np.zeros(ls.n * bs)
        foffd = np.zeros(max(nnz.value, 1) * bs)
        check(self.ctx.h, lib().dfg_precond_get_factor(self.h, _p(fdiag), _p(foffd)), "dfg_precond_get_factor")
        return fdiag, foffd[: nnz.value * bs]

    _close_order = 1

    def close(self):
        if getattr(self, "h", None):
            if self.ctx.h:
                lib().dfg_precond_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class LinearSystemPreconditioner:
    """LsSol::CLinearSystemPreconditioner (preconditioner.h:115-145): the
    ILinearSystemPreconditioner_Sol adapter the reference's own Solve_PCG drives."""

    def __init__(self, ls: LinearSystemField, prec: PreconditionerILU):
        self.ls, self.prec = ls, prec

    def GetTmpVectorArySize(self):
        return self.ls.GetTmpVectorArySize()

    def ReSizeTmpVecSolver(self, n):
        return self.ls.ReSizeTmpVecSolver(n)

    def DOT(self, a, b):
        return self.ls.DOT(a, b)

    def COPY(self, a, b):
        return self.ls.COPY(a, b)

    def SCAL(self, al, a):
        return self.ls.SCAL(al, a)

    def AXPY(self, al, a, b):
        return self.ls.AXPY(al, a, b)

    def MATVEC(self, al, a, be, b):
        return self.ls.MATVEC(al, a, be, b)

    def SolvePrecond(self, iv):
        return self.prec.SolvePrecond(self.ls, iv)


# ---------------------------------------------------------------- element routines

def AddLinSys_Poisson(ls: LinearSystemField, alpha: float, source: float):
    check(ls.ctx.h, lib().dfg_assemble_poisson(ls.h, alpha, source), "dfg_assemble_poisson")


def AddLinSys_Diffusion(dt: float, gamma: float, ls: LinearSystemField, rho: float, alpha: float, source: float):
    check(ls.ctx.h, lib().dfg_assemble_diffusion(ls.h, dt, gamma, rho, alpha, source), "dfg_assemble_diffusion")


def AddLinSys_LinearSolid2D_Static(ls: LinearSystemField, lam: float, myu: float, rho: float, g_x: float, g_y: float):
    check(ls.ctx.h, lib().dfg_assemble_solid2d(ls.h, lam, myu, rho, g_x, g_y), "dfg_assemble_solid2d")


def AddLinSys_LinearSolid3D_Static(ls: LinearSystemField, lam: float, myu: float, rho: float,
                                   g_x: float, g_y: float, g_z: float):
    check(ls.ctx.h, lib().dfg_assemble_solid3d(ls.h, lam, myu, rho, g_x, g_y, g_z), "dfg_assemble_solid3d")


# ---------------------------------------------------------------- solvers

def Solve_PCG(conv_ratio: float, iteration: int, ls: LinearSystemField, prec: PreconditionerILU):
    """LsSol::Solve_PCG (src/ls/solver_ls_iter.cpp:100-172), device-resident.
    Returns (converged, achieved ratio, 0-based iteration)."""
    c = ctypes.c_double(conv_ratio)
    it = ctypes.c_uint(iteration)
    st = lib().dfg_solve_pcg(ls.h, prec.h, ctypes.byref(c), ctypes.byref(it))
    if st not in (capi.DFG_OK, capi.DFG_NOT_CONVERGED):
        check(ls.ctx.h, st, "dfg_solve_pcg")
    return st == capi.DFG_OK, c.value, it.value


def Solve_PCG_Mixed(conv_ratio: float, iteration: int, ls: LinearSystemField, prec: PreconditionerILU):
    """FP32 factor / sweeps / SpMV inside FP64 refinement.  Returns
    (converged, true relative residual, inner iterations, refinement points)."""
    c = ctypes.c_double(conv_ratio)
    it = ctypes.c_uint(iteration)
    outer = ctypes.c_uint(0)
    st = lib().dfg_solve_pcg_mixed(ls.h, prec.h, ctypes.byref(c), ctypes.byref(it), ctypes.byref(outer))
    if st not in (capi.DFG_OK, capi.DFG_NOT_CONVERGED):
        check(ls.ctx.h, st, "dfg_solve_pcg_mixed")
    return st == capi.DFG_OK, c.value, it.value, outer.value


def Solve_PCG_ex(conv_ratio: float, iteration: int, ls: LinearSystemField, prec: PreconditionerILU,
                 mode: str = "fp64", target_true: bool = False):
    """dfg_solve_pcg_ex: mode "fp64" (plain), "mixed" (FP32 factor, sweeps, SpMV
    and vectors inside FP64 refinement) or "fp32f" (FP32 factor and sweeps,
    FP64 SpMV and vectors).  With target_true the true relative residual must
    also reach the tolerance.  Returns (converged, ratio, iterations, refinements)."""
    c = ctypes.c_double(conv_ratio)
    it = ctypes.c_uint(iteration)
    refin = ctypes.c_uint(0)
    st = lib().dfg_solve_pcg_ex(ls.h, prec.h, capi.MODES[mode], 1 if target_true else 0, ctypes.byref(c),
                                ctypes.byref(it), ctypes.byref(refin))
    if st not in (capi.DFG_OK, capi.DFG_NOT_CONVERGED):
        check(ls.ctx.h, st, "dfg_solve_pcg_ex")
    return st == capi.DFG_OK, c.value, it.value, refin.value


def Solve_PBiCGSTAB(conv_ratio: float, iteration: int, ls: LinearSystemField, prec: PreconditionerILU,
                    mode: str = "fp64"):
    """LsSol::Solve_PBiCGSTAB (src/ls/solver_ls_iter.cpp:291-408), device-resident,
    FP64 (other modes are rejected).  Returns (converged, ratio, 1-based
    iteration); when not converged the ratio is the tolerance given, as in the
    reference."""
    c = ctypes.c_double(conv_ratio)
    it = ctypes.c_uint(iteration)
    st = lib().dfg_solve_pbicgstab(ls.h, prec.h, capi.MODES[mode], ctypes.byref(c), ctypes.byref(it))
    if st not in (capi.DFG_OK, capi.DFG_NOT_CONVERGED):
        check(ls.ctx.h, st, "dfg_solve_pbicgstab")
    return st == capi.DFG_OK, c.value, it.value


def Solve_PBiCGSTAB_reference_loop(conv_ratio: float, iteration: int, lsp: LinearSystemPreconditioner):
    """The reference's Solve_PBiCGSTAB control flow (solver_ls_iter.cpp:291-408)
    over the ILinearSystemPreconditioner_Sol virtuals (the strict drop-in).
    Returns (the reference's return value, ratio, iteration)."""
    tol, mx = conv_ratio, iteration
    if lsp.GetTmpVectorArySize() < 7:
        lsp.ReSizeTmpVecSolver(7)
    ix, ir = -2, -1
    i_s, iMs, iAMs, ip, iMp, iAMp, ir2 = 0, 1, 2, 3, 4, 5, 6
    sq0 = lsp.DOT(ir, ir)
    if sq0 < 1.0e-60:
        return True, float(np.sqrt(sq0)), 0
    inv0 = 1.0 / sq0
    lsp.SCAL(0.0, ix)
    lsp.COPY(ir, ir2)
    lsp.COPY(ir, ip)
    for it in range(1, mx):
        lsp.COPY(ip, iMp)
        lsp.SolvePrecond(iMp)
        r_r2 = lsp.DOT(ir, ir2)
        lsp.MATVEC(1.0, iMp, 0.0, iAMp)
        alpha = r_r2 / lsp.DOT(iAMp, ir2)
        lsp.COPY(ir, i_s)
        lsp.AXPY(-alpha, iAMp, i_s)
        lsp.COPY(i_s, iMs)
        lsp.SolvePrecond(iMs)
        lsp.MATVEC(1.0, iMs, 0.0, iAMs)
        den = lsp.DOT(iAMs, iAMs)
        omega = lsp.DOT(i_s, iAMs) / den
        lsp.AXPY(alpha, iMp, ix)
        lsp.AXPY(omega, iMs, ix)
        lsp.COPY(i_s, ir)
        lsp.AXPY(-omega, iAMs, ir)
        sq = lsp.DOT(ir, ir)
        if sq * inv0 < tol * tol:
            return True, float(np.sqrt(sq * inv0)), it
        beta = lsp.DOT(ir, ir2) * alpha / (r_r2 * omega)
        lsp.SCAL(beta, ip)
        lsp.AXPY(1.0, ir, ip)
        lsp.AXPY(-beta * omega, iAMp, ip)
    return True, tol, mx


def Solve_PCG_reference_loop(conv_ratio: float, iteration: int, lsp: LinearSystemPreconditioner):
    """The reference's Solve_PCG control flow (solver_ls_iter.cpp:100-172)
    written against the ILinearSystemPreconditioner_Sol virtuals: this is how
    the unmodified reference solver drives the GPU system through the strict
    drop-in (one host round trip per DOT)."""
    tol, mx = conv_ratio, iteration
    if lsp.GetTmpVectorArySize() < 2:
        lsp.ReSizeTmpVecSolver(2)
    ix, ir, ip, iz = -2, -1, 0, 1
    lsp.SCAL(0.0, ix)
    s0 = lsp.DOT(ir, ir)
    if s0 < 1.0e-30:
        return True, 0.0, 0
    inv0 = 1.0 / s0
    lsp.COPY(ir, iz)
    lsp.SolvePrecond(iz)
    lsp.COPY(iz, ip)
    rz = lsp.DOT(ir, iz)
    for it in range(mx):
        lsp.MATVEC(1.0, ip, 0.0, iz)
        alpha = rz / lsp.DOT(ip, iz)
        lsp.AXPY(-alpha, iz, ir)
        lsp.AXPY(alpha, ip, ix)
        sq = lsp.DOT(ir, ir)
        if sq * inv0 < tol * tol:
            return True, float(np.sqrt(sq * inv0)), it
        lsp.COPY(ir, iz)
        lsp.SolvePrecond(iz)
        rz_new = lsp.DOT(ir, iz)
        beta = rz_new / rz
        rz = rz_new
        lsp.SCAL(beta, ip)
        lsp.AXPY(1.0, iz, ip)
    sq = lsp.DOT(ir, ir)
    return False, float(np.sqrt(sq * inv0)), mx


def profile_kernels(ls: LinearSystemField, prec: PreconditionerILU, mode: str = "fp64", reps: int = 20):
    """Per-launch device time (ms) of the kernels of one PCG iteration and the
    algorithmic bytes of the SpMV and the two sweeps."""
    ms = np.zeros(6)
    by = np.zeros(3)
    m = capi.MODES[mode]
    check(ls.ctx.h, lib().dfg_profile_kernels(ls.h, prec.h, m, reps, _p(ms), _p(by)), "dfg_profile_kernels")
    names = ["spmv", "sweep_fwd", "sweep_bwd", "update_rx", "rz_beta", "update_p"]
    return dict(zip(names, ms.tolist())), dict(zip(names[:3], by.tolist()))
