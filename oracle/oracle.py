"""Python driver for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/_build/libdfg_oracle.so (the C restatement in dfg_oracle.c,
built by ``make -C oracle port``) and runs the whole hot path of the
reference on a ``delfem_gb300.meshgen.Problem``: pattern, assembly,
extra loads, Dirichlet finalize, ILU(k) (k = 0 by default), PCG.  Only tests/, the smoke test
and bench.py's CPU-baseline leg import this module; the product never does.

``run_reference_harness`` executes the reference itself (oracle/_ref,
compiled from the reference sources) on the same problem; it exists only
where that build exists.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdfg_oracle.so")
HARNESS = os.path.join(HERE, "_ref", "ref_harness")

_lib = None

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double


def build() -> None:
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)


def reference_dir() -> str:
    """Where the reference checkout is looked for: DFG_REFERENCE_DIR when set,
    else the default the Makefile holds (``make refdir``)."""
    d = os.environ.get("DFG_REFERENCE_DIR")
    if d:
        return d
    r = subprocess.run(["make", "-s", "--no-print-directory", "-C", HERE, "refdir"], capture_output=True, text=True)
    return r.stdout.strip()


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.dfo_pattern.restype = ctypes.c_long
        L.dfo_pattern.argtypes = [_I, _I, _I, _P, _P, _P]
        L.dfo_diaind.argtypes = [_I, _P, _P, _P]
        for nm in ("dfo_assemble_poisson2d", "dfo_assemble_poisson3d"):
            getattr(L, nm).argtypes = [_I, _P, _P, _I, _P, _P, _P, _D, _D, _P, _P, _P, _P]
        L.dfo_assemble_diffusion2d.argtypes = [_I, _P, _P, _I, _P, _P, _P, _D, _D, _D, _D, _D, _P, _P, _P, _P, _P]
        L.dfo_assemble_solid2d.argtypes = [_I, _P, _P, _I, _P, _P, _P, _D, _D, _D, _D, _D, _P, _P, _P, _P]
        L.dfo_assemble_solid3d.argtypes = [_I, _P, _P, _I, _P, _P, _P, _D, _D, _D, _D, _D, _D, _P, _P, _P, _P]
        L.dfo_finalize.restype = _D
        L.dfo_finalize.argtypes = [_I, _I, _P, _P, _P, _P, _P, _P]
        L.dfo_ilu0.argtypes = [_I, _I, _P, _P, _P, _P, _P]
        L.dfo_forward.argtypes = [_I, _I, _P, _P, _P, _P, _P, _P]
        L.dfo_backward.argtypes = [_I, _I, _P, _P, _P, _P, _P]
        L.dfo_matvec.argtypes = [_I, _I, _P, _P, _P, _P, _D, _P, _D, _P]
        L.dfo_pcg.argtypes = [_I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                              ctypes.POINTER(_D), ctypes.POINTER(ctypes.c_uint), _P]
        L.dfo_pcg_f.argtypes = [_I, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                ctypes.POINTER(_D), ctypes.POINTER(ctypes.c_uint), _P]
        L.dfo_bicgstab.argtypes = L.dfo_pcg_f.argtypes
        L.dfo_ilu_pattern.restype = ctypes.c_long
        L.dfo_ilu_pattern.argtypes = [_I, _P, _P, _I, _P, _P, ctypes.c_long]
        L.dfo_ilu_init.argtypes = [_I, _I, _P, _P, _P, _P, _P, _P, _P, _P]
        L.dfo_now.restype = _D
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def pattern(nnode: int, conn: np.ndarray):
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    L = lib()
    nnz = L.dfo_pattern(nnode, conn.shape[0], conn.shape[1], _p(conn), None, None)
    if nnz < 0:
        raise ValueError("bad connectivity")
    rowptr = np.zeros(nnode + 1, dtype=np.int32)
    colind = np.zeros(max(nnz, 1), dtype=np.int32)
    L.dfo_pattern(nnode, conn.shape[0], conn.shape[1], _p(conn), _p(rowptr), _p(colind))
    return rowptr, colind[:nnz]


def diaind(rowptr, colind):
    n = rowptr.size - 1
    d = np.zeros(n, dtype=np.int32)
    lib().dfo_diaind(n, _p(rowptr), _p(colind), _p(d))
    return d


def ilu_pattern(rowptr, colind, fill_level: int):
    """Block pattern (rowptr_f, colind_f) of the ILU(fill_level) factor."""
    n = rowptr.size - 1
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    colind = np.ascontiguousarray(colind if colind.size else np.zeros(1, np.int32), dtype=np.int32)
    cap = max(2 * int(rowptr[-1]), 1)
    while True:
        rp = np.zeros(n + 1, dtype=np.int32)
        ci = np.zeros(cap, dtype=np.int32)
        nz = lib().dfo_ilu_pattern(n, _p(rowptr), _p(colind), fill_level, _p(rp), _p(ci), cap)
        if nz <= cap:
            return rp, ci[:nz]
        cap = nz


def assemble(p, rowptr, colind):
    """Returns (diag, offd, res) before loads / Dirichlet finalize."""
    from delfem_gb300 import meshgen as mg
    n, b = p.nnode, p.b
    bs = b * b
    diag = np.zeros(n * bs)
    offd = np.zeros(max(colind.size, 1) * bs)
    res = np.zeros(n * b)
    L = lib()
    coords = np.ascontiguousarray(p.coords, dtype=np.float64)
    conn = np.ascontiguousarray(p.conn, dtype=np.int32)
    coef = None if p.coef is None else np.ascontiguousarray(p.coef, dtype=np.float64)
    u = None if p.u is None else np.ascontiguousarray(p.u, dtype=np.float64)
    v = None if p.v is None else np.ascontiguousarray(p.v, dtype=np.float64)
    P = [float(x) for x in p.params]
    common = (n, _p(rowptr), _p(colind), p.nelem, _p(conn), _p(coords), _p(coef))
    if p.kind == mg.POISSON2D:
        rc = L.dfo_assemble_poisson2d(*common, P[0], P[1], _p(u), _p(diag), _p(offd), _p(res))
    elif p.kind == mg.POISSON3D:
        rc = L.dfo_assemble_poisson3d(*common, P[0], P[1], _p(u), _p(diag), _p(offd), _p(res))
    elif p.kind == mg.DIFFUSION2D:
        rc = L.dfo_assemble_diffusion2d(*common, P[0], P[1], P[2], P[3], P[4], _p(u), _p(v),
                                        _p(diag), _p(offd), _p(res))
    elif p.kind == mg.SOLID2D:
        rc = L.dfo_assemble_solid2d(*common, P[0], P[1], P[2], P[3], P[4], _p(u),
                                    _p(diag), _p(offd), _p(res))
    elif p.kind == mg.SOLID3D:
        rc = L.dfo_assemble_solid3d(*common, P[0], P[1], P[2], P[3], P[4], P[5], _p(u),
                                    _p(diag), _p(offd), _p(res))
    else:
        raise ValueError(p.kind)
    if rc != 0:
        raise ValueError("assembly failed")
    return diag, offd[: colind.size * bs], res


def solve(p, tol=None, maxit=None, stop_after_ilu=False, fill_level: int = 0, solver: str = "pcg") -> dict:
    """The reference's whole path on the CPU with an ILU(fill_level)
    preconditioner and Solve_PCG or Solve_PBiCGSTAB; returns every
    intermediate."""
    L = lib()
    t0 = L.dfo_now()
    rowptr, colind = pattern(p.nnode, p.conn)
    n, b = p.nnode, p.b
    bs = b * b
    diag, offd, res = assemble(p, rowptr, colind)
    if p.load is not None:
        res = res + np.asarray(p.load, dtype=np.float64)
    t1 = L.dfo_now()
    bc = np.ascontiguousarray(p.bcflag, dtype=np.int32)
    offd_c = np.ascontiguousarray(offd) if offd.size else np.zeros(1)
    norm_res = L.dfo_finalize(n, b, _p(rowptr), _p(colind), _p(bc), _p(diag), _p(offd_c), _p(res))
    offd = offd_c[: colind.size * bs]
    rhs = res.copy()
    dind = diaind(rowptr, colind)
    t2 = L.dfo_now()
    if fill_level == 0:
        rowptr_f, colind_f, dind_f = rowptr, colind, dind
        fdiag = diag.copy()
        foffd = offd.copy() if offd.size else np.zeros(1)
    else:
        rowptr_f, colind_f = ilu_pattern(rowptr, colind, fill_level)
        dind_f = diaind(rowptr_f, colind_f)
        fdiag = np.zeros(n * bs)
        foffd = np.zeros(max(colind_f.size, 1) * bs)
        offd_a = offd if offd.size else np.zeros(1)
        cf = colind_f if colind_f.size else np.zeros(1, np.int32)
        if L.dfo_ilu_init(n, b, _p(rowptr), _p(colind), _p(diag), _p(offd_a), _p(rowptr_f), _p(cf),
                          _p(fdiag), _p(foffd)) != 0:
            raise ValueError("A's pattern is not inside the factor's")
    cf = colind_f if colind_f.size else np.zeros(1, np.int32)
    ilu_rc = L.dfo_ilu0(n, b, _p(rowptr_f), _p(cf), _p(dind_f), _p(fdiag), _p(foffd))
    t3 = L.dfo_now()
    out = dict(n=n, b=b, nnz=colind.size, rowptr=rowptr, colind=colind, diaind=dind,
               diag=diag, offd=offd, rhs=rhs, norm_res=norm_res, ilu_rc=ilu_rc, fill_level=fill_level,
               rowptr_f=rowptr_f, colind_f=colind_f, diaind_f=dind_f,
               fdiag=fdiag, foffd=foffd[: colind_f.size * bs], t_assemble=t1 - t0, t_ilu=t3 - t2)
    if stop_after_ilu:
        return out
    out.update(bicgstab(out, p.tol if tol is None else tol, p.maxit if maxit is None else maxit)
               if solver == "bicgstab" else {})
    if solver == "bicgstab":
        return out
    r = rhs.copy()
    x = np.zeros(n * b)
    work = np.zeros(2 * n * b)
    conv = ctypes.c_double(p.tol if tol is None else tol)
    it = ctypes.c_uint(p.maxit if maxit is None else maxit)
    offd_a = offd if offd.size else np.zeros(1)
    t4 = L.dfo_now()
    ok = L.dfo_pcg_f(n, b, _p(rowptr), _p(colind), _p(diag), _p(offd_a), _p(rowptr_f), _p(cf), _p(dind_f),
                     _p(fdiag), _p(foffd), _p(r), _p(x), ctypes.byref(conv), ctypes.byref(it), _p(work))
    t5 = L.dfo_now()
    out.update(x=x, conv=conv.value, iter=it.value, converged=bool(ok), t_pcg=t5 - t4)
    return out


def bicgstab(out: dict, tol: float, maxit: int, rhs=None, diag=None, offd=None, x0=None) -> dict:
    """Solve_PBiCGSTAB on the system and factor in ``out`` (a ``solve(...,
    stop_after_ilu=True)`` result); the matrix and right-hand side may be
    replaced (e.g. by a non-symmetric one with the same pattern, factorised
    by the caller into out["fdiag"] / out["foffd"])."""
    L = lib()
    n, b = out["n"], out["b"]
    diag = out["diag"] if diag is None else diag
    offd = out["offd"] if offd is None else offd
    r = np.array(out["rhs"] if rhs is None else rhs, dtype=np.float64, copy=True)
    x = np.zeros(n * b) if x0 is None else np.array(x0, dtype=np.float64, copy=True)
    work = np.zeros(7 * n * b)
    conv = ctypes.c_double(tol)
    it = ctypes.c_uint(maxit)
    offd_a = offd if offd.size else np.zeros(1)
    cf = out["colind_f"] if out["colind_f"].size else np.zeros(1, np.int32)
    fo = out["foffd"] if out["foffd"].size else np.zeros(1)
    t0 = L.dfo_now()
    ok = L.dfo_bicgstab(n, b, _p(out["rowptr"]), _p(out["colind"]), _p(diag), _p(offd_a), _p(out["rowptr_f"]),
                        _p(cf), _p(out["diaind_f"]), _p(out["fdiag"]), _p(fo), _p(r), _p(x), ctypes.byref(conv),
                        ctypes.byref(it), _p(work))
    return dict(x=x, conv=conv.value, iter=it.value, converged=bool(ok), t_solve=L.dfo_now() - t0, r=r)


def factor(out: dict, diag, offd):
    """ILU factor of another matrix on the pattern of ``out`` (same fill)."""
    L = lib()
    n, b = out["n"], out["b"]
    bs = b * b
    fdiag = np.zeros(n * bs)
    foffd = np.zeros(max(out["colind_f"].size, 1) * bs)
    cf = out["colind_f"] if out["colind_f"].size else np.zeros(1, np.int32)
    offd_a = offd if offd.size else np.zeros(1)
    if L.dfo_ilu_init(n, b, _p(out["rowptr"]), _p(out["colind"] if out["colind"].size else np.zeros(1, np.int32)),
                      _p(diag), _p(offd_a), _p(out["rowptr_f"]), _p(cf), _p(fdiag), _p(foffd)) != 0:
        raise ValueError("pattern mismatch")
    rc = L.dfo_ilu0(n, b, _p(out["rowptr_f"]), _p(cf), _p(out["diaind_f"]), _p(fdiag), _p(foffd))
    return fdiag, foffd[: out["colind_f"].size * bs], rc


def matvec(n, b, rowptr, colind, diag, offd, x, alpha=1.0, beta=0.0, y=None):
    y = np.zeros(n * b) if y is None else y.copy()
    offd_a = offd if offd.size else np.zeros(1)
    lib().dfo_matvec(n, b, _p(rowptr), _p(colind), _p(diag), _p(offd_a), alpha, _p(x), beta, _p(y))
    return y


def precond(n, b, rowptr, colind, dind, fdiag, foffd, r):
    z = np.array(r, dtype=np.float64, copy=True)
    fo = foffd if foffd.size else np.zeros(1)
    lib().dfo_forward(n, b, _p(rowptr), _p(colind), _p(dind), _p(fdiag), _p(fo), _p(z))
    lib().dfo_backward(n, b, _p(rowptr), _p(colind), _p(dind), _p(fo), _p(z))
    return z


def true_residual(out: dict, x: np.ndarray) -> float:
    """||b - A x|| / ||b|| in FP64 with the assembled (post-BC) matrix."""
    Ax = matvec(out["n"], out["b"], out["rowptr"], out["colind"], out["diag"], out["offd"], x)
    bn = float(np.linalg.norm(out["rhs"]))
    return float(np.linalg.norm(out["rhs"] - Ax)) / (bn if bn > 0 else 1.0)


def harness_available() -> bool:
    return os.path.exists(HARNESS)


def run_reference_harness(p, fill_level: int = 0, solver: str = "pcg") -> dict:
    """Runs the reference code itself (oracle/_ref/ref_harness) on ``p`` with
    an ILU preconditioner of the given fill level and Solve_PCG ("pcg") or
    Solve_PBiCGSTAB ("bicgstab")."""
    from delfem_gb300 import meshgen as mg
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "p.bin"), os.path.join(td, "r.bin")
        mg.write_problem(p, fi)
        subprocess.run([HARNESS, fi, fo, str(fill_level), solver], check=True, stdout=subprocess.DEVNULL)
        return mg.read_result(fo)


def make_problem(spec: tuple):
    """A generated problem from a picklable spec: ("factory", kwargs) names a
    meshgen problem factory; ("stream2d" | "stream3d", kwargs with `index`)
    one request of a serving stream."""
    from delfem_gb300 import meshgen as mg
    name, kw = spec
    kw = dict(kw)
    if name in ("stream2d", "stream3d"):
        idx = kw.pop("index")
        items = mg.serve_stream_2d(**kw) if name == "stream2d" else mg.serve_stream_3d(**kw)
        return items[idx].problem()
    return getattr(mg, name)(**kw)


def solve_digest(spec: tuple, fill_level: int = 0) -> dict:
    """solve() on make_problem(spec), returning SHA-256 digests of the large
    arrays (pattern as int32, assembled matrix, finalized right-hand side,
    ILU factor) with the iteration count, ratio and solution vector: for
    parity tests at sizes where hashing the arrays costs less than shipping
    them between processes.  Runs in a spawned worker."""
    import hashlib

    def h(a, dtype):
        return hashlib.sha256(np.ascontiguousarray(a, dtype=dtype).tobytes()).hexdigest()

    p = make_problem(spec)
    t0 = lib().dfo_now()
    out = solve(p, fill_level=fill_level)
    return dict(rowptr=h(out["rowptr"], np.int32), colind=h(out["colind"], np.int32),
                diag=h(out["diag"], np.float64), offd=h(out["offd"], np.float64), rhs=h(out["rhs"], np.float64),
                fdiag=h(out["fdiag"], np.float64), foffd=h(out["foffd"], np.float64), ilu_rc=int(out["ilu_rc"]),
                iter=int(out["iter"]), conv=float(out["conv"]), converged=bool(out["converged"]), x=out["x"],
                true_rel=true_residual(out, out["x"]), seconds=lib().dfo_now() - t0)
