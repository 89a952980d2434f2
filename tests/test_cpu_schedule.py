"""The host sweep scheduler (delfem_gb300/csrc/sched.cpp), executed by a
sequential CPU emulator of the GPU kernel's dependency decoding
(tests/cpu/sweep_emul.cpp): complete coverage, valid ring references, no
wait on a later range, and forward/backward results equal to the oracle's
substitutions up to summation order.  The level schedule of the
level-scheduled sweep (build_levels) is executed the same way, in the level
kernel's summation order."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

EMUL_SO = os.path.join(ROOT, "tests", "cpu", "_build", "libsweep_emul.so")


@pytest.fixture(scope="module")
def emul():
    os.makedirs(os.path.dirname(EMUL_SO), exist_ok=True)
    srcs = [os.path.join(ROOT, "tests", "cpu", "sweep_emul.cpp"), os.path.join(ROOT, "delfem_gb300", "csrc", "sched.cpp")]
    # (sched.cpp includes the CUDA runtime header for cudaStream_t only; no CUDA code runs)
    inc = [d for d in ("/usr/local/cuda/include",) if os.path.isdir(d)]
    subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", *[f"-I{d}" for d in inc], "-o", EMUL_SO, *srcs],
                   check=True)
    L = ctypes.CDLL(EMUL_SO)
    P = ctypes.c_void_p
    L.emul_sweep.argtypes = [ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, P, P, P]
    L.emul_solo_precond.argtypes = [ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.c_int, P, P, P, P, P]
    L.emul_solo_shape.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_longlong, P]
    L.emul_ilu_pattern.restype = ctypes.c_longlong
    L.emul_ilu_pattern.argtypes = [ctypes.c_int, P, P, ctypes.c_int, P, P, ctypes.c_longlong]
    return L


def _lib_ilu_pattern(emul, rowptr, colind, lev):
    n = rowptr.size - 1
    ci0 = colind if colind.size else np.zeros(1, np.int32)
    nz = emul.emul_ilu_pattern(n, _p(rowptr), _p(ci0), lev, None, None, -1)
    rp = np.zeros(n + 1, np.int32)
    ci = np.zeros(max(nz, 1), np.int32)
    assert emul.emul_ilu_pattern(n, _p(rowptr), _p(ci0), lev, _p(rp), _p(ci), nz) == nz
    return rp, ci[:nz]


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _problems():
    from delfem_gb300 import meshgen as mg
    return [mg.poisson2d_square(20, seed=3), mg.solid2d_cantilever(30, 12, seed=4), mg.solid3d_cube(6, seed=5),
            mg.poisson3d_cube(7, seed=6, coef_sigma=1.0)]


@pytest.mark.parametrize("idx", range(4))
@pytest.mark.parametrize("range_rows", [-1, 0, 1, 37, 256, 100000])
@pytest.mark.parametrize("R", [2, 8, 32])
def test_sweep_schedule(emul, oracle_lib, idx, range_rows, R):
    p = _problems()[idx]
    out = oracle_lib.solve(p, stop_after_ilu=True)
    n, b = out["n"], out["b"]
    rhs = np.random.default_rng(idx).standard_normal(n * b)
    fo = out["foffd"] if out["foffd"].size else np.zeros(1)
    # forward then backward through the emulator
    y = np.full(n * b, np.nan)
    info = np.zeros(8, dtype=np.int64)
    rc = emul.emul_sweep(n, b, _p(out["rowptr"]), _p(out["colind"]), 1, range_rows, R, _p(out["fdiag"]), _p(fo),
                         _p(rhs), _p(y), _p(info))
    assert rc == 0, f"forward schedule check failed with code {rc}"
    z = np.full(n * b, np.nan)
    rc = emul.emul_sweep(n, b, _p(out["rowptr"]), _p(out["colind"]), 0, range_rows, R, _p(out["fdiag"]), _p(fo),
                         _p(y), _p(z), _p(info))
    assert rc == 0, f"backward schedule check failed with code {rc}"
    ref = oracle_lib.precond(n, b, out["rowptr"], out["colind"], out["diaind"], out["fdiag"], out["foffd"], rhs)
    np.testing.assert_allclose(z, ref, rtol=1e-11, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("idx", range(4))
def test_sell_layout_matches_crs_product(emul, oracle_lib, idx):
    """The sliced-ELL copy covers every block once and its thread-per-row
    product repeats the CRS row-order sum bit for bit (g++ without FMA
    contraction on both sides)."""
    from conftest import bits
    p = _problems()[idx]
    out = oracle_lib.solve(p, stop_after_ilu=True)
    n, b = out["n"], out["b"]
    x = np.random.default_rng(10 + idx).standard_normal(n * b)
    ys, yc = np.zeros(n * b), np.zeros(n * b)
    info = np.zeros(4, dtype=np.int64)
    P = ctypes.c_void_p
    emul.emul_sell.argtypes = [ctypes.c_int, ctypes.c_int, P, P, P, P, P, P, P, P]
    od = out["offd"] if out["offd"].size else np.zeros(1)
    rc = emul.emul_sell(n, b, _p(out["rowptr"]), _p(out["colind"]), _p(out["diag"]), _p(od), _p(x), _p(ys), _p(yc),
                        _p(info))
    assert rc == 0
    assert info[0] == (n + 31) // 32
    assert np.array_equal(bits(ys), bits(yc))
    xr = oracle_lib.matvec(n, b, out["rowptr"], out["colind"], out["diag"], out["offd"], x)
    np.testing.assert_allclose(ys, xr, rtol=1e-12, atol=1e-14 * np.abs(xr).max())


def test_serving_schedule_has_fuller_steps(emul, oracle_lib):
    """The batched-launch schedule (range_rows -1: fullest steps) packs more
    rows per step than the single-solve choice on serving-like meshes."""
    from delfem_gb300 import meshgen as mg
    for p in (mg.rect_problem_2d(mg.SOLID2D, 20000, seed=3), mg.rect_problem_2d(mg.POISSON2D, 30000, seed=4)):
        out = oracle_lib.solve(p, stop_after_ilu=True)
        n, b = out["n"], out["b"]
        rhs = np.ones(n * b)
        fo = out["foffd"] if out["foffd"].size else np.zeros(1)
        fill = {}
        for rr in (-1, 0):
            y = np.full(n * b, np.nan)
            info = np.zeros(8, dtype=np.int64)
            assert emul.emul_sweep(n, b, _p(out["rowptr"]), _p(out["colind"]), 1, rr, 32, _p(out["fdiag"]), _p(fo),
                                   _p(rhs), _p(y), _p(info)) == 0
            fill[rr] = n / info[1]
        assert fill[-1] >= fill[0], fill
        assert fill[-1] > 20, fill


def _solo(emul, out, R, elem, stage_bytes, ch_max, rhs):
    n, b = out["n"], out["b"]
    fo = out["foffd"] if out["foffd"].size else np.zeros(1)
    z = np.full(n * b, np.nan)
    info = np.zeros(8, dtype=np.int64)
    rc = emul.emul_solo_precond(n, b, _p(out["rowptr"]), _p(out["colind"]), R, elem, stage_bytes, ch_max,
                                _p(out["fdiag"]), _p(fo), _p(rhs), _p(z), _p(info))
    return rc, z, info


@pytest.mark.parametrize("idx", range(4))
@pytest.mark.parametrize("R,stage,ch", [(16, 4096, 2), (256, 20000, 4), (512, 100000, 8), (64, 120000, 16)])
@pytest.mark.parametrize("elem", [4, 8])
def test_solo_schedule(emul, oracle_lib, idx, R, stage, ch, elem):
    """The one-CTA-per-solve schedules executed as k_solo.cu runs them,
    through their packed records and the server's storage orders: chunks
    that tile the steps in order (narrow levels sharing a chunk) within their
    bounds, ring references that the consuming level never overwrites,
    global references to rows of earlier
    levels at their storage positions, and a preconditioner apply equal to the
    oracle's substitutions up to rounding."""
    p = _problems()[idx]
    out = oracle_lib.solve(p, stop_after_ilu=True)
    n, b = out["n"], out["b"]
    rhs = np.random.default_rng(idx).standard_normal(n * b)
    rc, z, info = _solo(emul, out, R, elem, stage, ch, rhs)
    assert rc == 0, info
    # chunks may span narrow levels: at least the forward steps over ch_max
    assert info[4] + info[5] > 0 and info[6] >= (info[1] + ch - 1) // ch
    dind = oracle_lib.diaind(out["rowptr"], out["colind"])
    zref = oracle_lib.precond(n, b, out["rowptr"], out["colind"], dind, out["fdiag"], out["foffd"], rhs)
    np.testing.assert_allclose(z, zref, rtol=1e-12, atol=1e-13 * np.abs(zref).max())


def test_solo_schedule_ring_covers_2d_levels(emul, oracle_lib):
    """On a serving-sized 2D mesh a 128-step ring holds every dependency: a
    level's rows depend on the level before it only."""
    from delfem_gb300 import meshgen as mg
    p = mg.rect_problem_2d(mg.SOLID2D, 30000, seed=3)
    out = oracle_lib.solve(p, stop_after_ilu=True)
    rc, z, info = _solo(emul, out, 128, 4, 30000, 8, np.ones(out["n"] * out["b"]))
    assert rc == 0 and info[5] == 0 and info[4] > 0, info


def test_library_fill_pattern_matches_reference(emul):
    """The library's host ILU(k) pattern builder equals the reference's
    AddFracPtn output on every fixture of tests/golden/iluk/."""
    from conftest import golden_iluk_files, load_golden
    files = golden_iluk_files()
    assert files
    for f in files:
        _, ref = load_golden(f)
        rp, ci = _lib_ilu_pattern(emul, ref["rowptr"].astype(np.int32), ref["colind"].astype(np.int32),
                                  int(ref["fill_level"]))
        assert np.array_equal(rp, ref["rowptr_f"]) and np.array_equal(ci, ref["colind_f"]), f


@pytest.mark.parametrize("lev", [0, 1, 2, 3, -1])
def test_library_fill_pattern_matches_oracle(emul, oracle_lib, lev):
    from delfem_gb300 import meshgen as mg
    for p in (mg.poisson2d_square(15, seed=7), mg.solid2d_cantilever(12, 6, seed=8), mg.poisson3d_cube(4, seed=9)):
        rp, ci = oracle_lib.pattern(p.nnode, p.conn)
        a = _lib_ilu_pattern(emul, rp, ci, lev)
        b = oracle_lib.ilu_pattern(rp, ci, lev)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (p.name, lev)


@pytest.mark.parametrize("lev", [1, 2, -1])
@pytest.mark.parametrize("range_rows", [-1, 0, 37])
def test_sweep_schedule_on_fill_pattern(emul, oracle_lib, lev, range_rows):
    """Sweep schedules built on an ILU(k) factor pattern pass the same checks
    and reproduce the oracle's ILU(k) substitutions."""
    from delfem_gb300 import meshgen as mg
    p = mg.solid2d_cantilever(16, 7, seed=21, coef_sigma=0.5)
    out = oracle_lib.solve(p, stop_after_ilu=True, fill_level=lev)
    n, b = out["n"], out["b"]
    rp, ci, di = out["rowptr_f"], out["colind_f"], out["diaind_f"]
    rhs = np.random.default_rng(lev + 5).standard_normal(n * b)
    fo = out["foffd"] if out["foffd"].size else np.zeros(1)
    info = np.zeros(8, dtype=np.int64)
    y = np.full(n * b, np.nan)
    assert emul.emul_sweep(n, b, _p(rp), _p(ci), 1, range_rows, 8, _p(out["fdiag"]), _p(fo), _p(rhs), _p(y),
                           _p(info)) == 0
    z = np.full(n * b, np.nan)
    assert emul.emul_sweep(n, b, _p(rp), _p(ci), 0, range_rows, 8, _p(out["fdiag"]), _p(fo), _p(y), _p(z),
                           _p(info)) == 0
    ref = oracle_lib.precond(n, b, rp, ci, di, out["fdiag"], out["foffd"], rhs)
    np.testing.assert_allclose(z, ref, rtol=1e-11, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("dim,lev", [(2, 1), (2, 2), (2, -1), (3, 1), (3, 2)])
def test_library_fill_pattern_on_unstructured_meshes(emul, oracle_lib, dim, lev):
    """Delaunay meshes in random node order (irregular valences and fill)."""
    pytest.importorskip("scipy")
    from delfem_gb300 import meshgen as mg
    co, cn = mg.delaunay_mesh(400 if dim == 2 else 150, dim, seed=dim * 10 + lev)
    rp, ci = oracle_lib.pattern(co.shape[0], cn)
    a = _lib_ilu_pattern(emul, rp, ci, lev)
    b = oracle_lib.ilu_pattern(rp, ci, lev)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def _level_sweep(emul, n, b, rowptr, colind, forward, fdiag, foffd, vin):
    P = ctypes.c_void_p
    emul.emul_level_sweep.argtypes = [ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int, P, P, P, P, P]
    out = np.zeros(max(n * b, 1))
    info = np.zeros(4, dtype=np.int64)
    rc = emul.emul_level_sweep(n, b, _p(rowptr), _p(colind if colind.size else np.zeros(1, np.int32)), forward,
                               _p(fdiag if fdiag.size else np.zeros(1)), _p(foffd if foffd.size else np.zeros(1)),
                               _p(vin if vin.size else np.zeros(1)), _p(out), _p(info))
    return rc, out[:n * b], info


@pytest.mark.parametrize("idx", range(4))
@pytest.mark.parametrize("lev", [0, 1])
def test_level_schedule(emul, oracle_lib, idx, lev):
    """The level schedule (sched.cpp build_levels) on ILU(0) and ILU(1)
    factors: a permutation grouped by level, dependencies in earlier levels,
    longest-path levels, and forward then backward substitution in the level
    kernel's summation order equal to the oracle's preconditioner apply."""
    p = _problems()[idx]
    out = oracle_lib.solve(p, stop_after_ilu=True, fill_level=lev)
    n, b = out["n"], out["b"]
    rp, ci = out["rowptr_f"], out["colind_f"]
    rhs = np.random.default_rng(40 + idx).standard_normal(n * b)
    rc, y, info_f = _level_sweep(emul, n, b, rp, ci, 1, out["fdiag"], out["foffd"], rhs)
    assert rc == 0, f"forward level schedule check failed with code {rc}"
    rc, z, info_b = _level_sweep(emul, n, b, rp, ci, 0, out["fdiag"], out["foffd"], y)
    assert rc == 0, f"backward level schedule check failed with code {rc}"
    assert 1 <= info_f[0] <= n and 1 <= info_b[0] <= n
    ref = oracle_lib.precond(n, b, rp, ci, out["diaind_f"], out["fdiag"], out["foffd"], rhs)
    np.testing.assert_allclose(z, ref, rtol=1e-11, atol=1e-12 * np.abs(ref).max())


def test_level_schedule_shapes(emul):
    """Hand-made patterns: a chain (one row per level), a diagonal matrix
    (one level), a long row (more than 32 dependencies, so several entries per
    lane) and an empty system (no level)."""
    def run(rows, n, b=1):
        rp = np.zeros(n + 1, np.int32)
        rp[1:] = np.cumsum([len(r) for r in rows])
        ci = np.array([c for r in rows for c in sorted(r)], dtype=np.int32)
        rng = np.random.default_rng(n)
        fdiag = np.tile(np.eye(b).ravel(), n) * 0.5
        foffd = rng.standard_normal(ci.size * b * b) * 0.01
        vin = rng.standard_normal(n * b)
        rc, y, info = _level_sweep(emul, n, b, rp, ci, 1, fdiag, foffd, vin)
        assert rc == 0
        # plain forward substitution (unit lower factor, then the diagonal inverse)
        yr = np.zeros(n * b)
        for i in range(n):
            acc = vin[i * b:(i + 1) * b].copy()
            for k in range(rp[i], rp[i + 1]):
                j = ci[k]
                if j < i:
                    acc -= foffd[k * b * b:(k + 1) * b * b].reshape(b, b) @ yr[j * b:(j + 1) * b]
            yr[i * b:(i + 1) * b] = fdiag[i * b * b:(i + 1) * b * b].reshape(b, b) @ acc
        np.testing.assert_allclose(y, yr, rtol=1e-13, atol=1e-14)
        return info
    n = 50
    chain = [[i - 1, i + 1] if 0 < i < n - 1 else ([1] if i == 0 else [n - 2]) for i in range(n)]
    assert run(chain, n)[0] == n
    assert run([[] for _ in range(n)], n)[:2].tolist() == [1, n]
    wide = [[j for j in range(100) if j != i] if i == 99 else ([99] if i < 99 else []) for i in range(101)]
    info = run(wide, 101, b=3)
    assert info[0] == 2 and info[1] == 100
    assert run([], 0)[0] == 0


@pytest.mark.parametrize("b", [1, 2, 3])
@pytest.mark.parametrize("maxe", [4, 8, 16])
@pytest.mark.parametrize("elem", [4, 8])
@pytest.mark.parametrize("forward", [0, 1])
def test_solo_shape(emul, b, maxe, elem, forward):
    """The one-CTA sweep's per-class launch shape within one SM's shared
    memory (GB300: 232,448 bytes a CTA may opt into, less the 4 KB the
    server leaves): a power-of-two ring of at most 512 steps, 1-16 steps per
    chunk, at least two stages and at least four for chunks above 8 steps, a
    stage that holds a full chunk's records, and the kernel's own byte count
    (k_sweep.h solo_smem_bytes) inside the budget."""
    budget = 232448 - 4096
    out = np.zeros(5, dtype=np.int64)
    emul.emul_solo_shape(b, maxe, elem, forward, budget, _p(out))
    R, ch, rec_stage, ns, smem = (int(v) for v in out)
    assert 16 <= R <= 512 and R & (R - 1) == 0
    assert 1 <= ch <= 16 and ns >= (4 if ch > 8 else 2), (ch, ns)
    rec1 = 16 + 128 + maxe * 128 + maxe * 32 * b * b * elem + (32 * b * b * elem if forward else 0)
    assert rec_stage == ch * rec1
    assert 0 < smem <= budget
