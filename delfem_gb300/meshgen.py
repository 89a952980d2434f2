"""Seeded synthetic meshes and load cases for the DelFEM hot path.

These stand in for the meshes the reference's own programs build through
``Msh::IMesh`` (include/delfem/mesh_interface.h:58-74): node coordinates in
``GetCoord`` order (which is the DOF order and therefore the ILU ordering)
and one element array of P1 triangles or tetrahedra.

* ``tri_grid``  -- nx x ny cells, each split along its (i,j)-(i+1,j+1)
  diagonal into two counter-clockwise triangles; interior nodes jittered by
  U(-f*h, f*h) per axis.  Node id = j*(nx+1)+i, element id = 2*(j*nx+i)+t.
* ``tet_grid``  -- nx x ny x nz hexes, each split into the 6 Kuhn tetrahedra
  around its (0,0,0)-(1,1,1) diagonal, positively oriented.
  Node id = (k*(ny+1)+j)*(nx+1)+i.

Problem kinds match the element routines of the reference:
POISSON2D (eqn_poisson.cpp:49), POISSON3D (:249), DIFFUSION2D
(eqn_diffusion.cpp:240), SOLID2D (eqn_linear_solid2d.cpp:505),
SOLID3D (eqn_linear_solid3d.cpp:241).
"""
from __future__ import annotations

import dataclasses
import itertools
import struct

import numpy as np

POISSON2D, POISSON3D, DIFFUSION2D, SOLID2D, SOLID3D = 1, 2, 3, 4, 5
KIND_NAMES = {POISSON2D: "poisson2d", POISSON3D: "poisson3d", DIFFUSION2D: "diffusion2d",
              SOLID2D: "solid2d", SOLID3D: "solid3d"}
BLOCK = {POISSON2D: 1, POISSON3D: 1, DIFFUSION2D: 1, SOLID2D: 2, SOLID3D: 3}
NDIM = {POISSON2D: 2, POISSON3D: 3, DIFFUSION2D: 2, SOLID2D: 2, SOLID3D: 3}


@dataclasses.dataclass
class Problem:
    kind: int
    coords: np.ndarray          # (nnode, ndim) float64
    conn: np.ndarray            # (nelem, nnoel) int32
    params: np.ndarray          # (8,) float64, meaning per kind (see ``params_doc``)
    bcflag: np.ndarray          # (nnode*b,) int32, 1 = Dirichlet DOF
    coef: np.ndarray | None = None   # (nelem,) per-element multiplier
    load: np.ndarray | None = None   # (nnode*b,) extra nodal load added to the residual
    u: np.ndarray | None = None      # (nnode*b,) current field value
    v: np.ndarray | None = None      # (nnode*b,) current field velocity (diffusion only)
    tol: float = 1e-8
    maxit: int = 20000
    name: str = ""

    @property
    def b(self) -> int:
        return BLOCK[self.kind]

    @property
    def nnode(self) -> int:
        return self.coords.shape[0]

    @property
    def nelem(self) -> int:
        return self.conn.shape[0]

    @property
    def ndof(self) -> int:
        return self.nnode * self.b


def params_doc(kind: int) -> str:
    return {
        POISSON2D: "alpha, source",
        POISSON3D: "alpha, source",
        DIFFUSION2D: "rho, alpha, source, gamma, dt",
        SOLID2D: "lambda, myu, rho, g_x, g_y",
        SOLID3D: "lambda, myu, rho, g_x, g_y, g_z",
    }[kind]


def lame(E: float, nu: float) -> tuple[float, float]:
    """Plane-strain / 3D Lame constants (the raw 2D P1 kernel is plane strain
    when given the 3D lambda, eqn_linear_solid2d.cpp:564-571)."""
    lam = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    myu = E / (2.0 * (1.0 + nu))
    return lam, myu


def tri_grid(nx: int, ny: int, lx: float = 1.0, ly: float = 1.0, jitter: float = 0.0,
             rng: np.random.Generator | None = None) -> tuple[np.ndarray, np.ndarray]:
    hx, hy = lx / nx, ly / ny
    i, j = np.meshgrid(np.arange(nx + 1), np.arange(ny + 1), indexing="xy")
    x = (i * hx).astype(np.float64).ravel()
    y = (j * hy).astype(np.float64).ravel()
    if jitter > 0.0:
        rng = rng or np.random.default_rng(0)
        interior = ((i > 0) & (i < nx) & (j > 0) & (j < ny)).ravel()
        dx = rng.uniform(-jitter * hx, jitter * hx, size=x.shape)
        dy = rng.uniform(-jitter * hy, jitter * hy, size=y.shape)
        x = np.where(interior, x + dx, x)
        y = np.where(interior, y + dy, y)
    coords = np.stack([x, y], axis=1)
    ci, cj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="xy")
    ci, cj = ci.ravel(), cj.ravel()
    n00 = cj * (nx + 1) + ci
    n10 = n00 + 1
    n01 = n00 + (nx + 1)
    n11 = n01 + 1
    t0 = np.stack([n00, n10, n11], axis=1)
    t1 = np.stack([n00, n11, n01], axis=1)
    conn = np.stack([t0, t1], axis=1).reshape(-1, 3).astype(np.int32)
    return coords, conn


_KUHN = None


def _kuhn_tets() -> np.ndarray:
    global _KUHN
    if _KUHN is None:
        tets = []
        for perm in itertools.permutations(range(3)):
            v = [0, 0, 0]
            verts = [tuple(v)]
            for a in perm:
                v[a] = 1
                verts.append(tuple(v))
            tets.append(verts)
        _KUHN = np.array(tets, dtype=np.int64)  # (6, 4, 3) local corner offsets
    return _KUHN


def tet_grid(nx: int, ny: int, nz: int, lx: float = 1.0, ly: float = 1.0, lz: float = 1.0,
             jitter: float = 0.0, rng: np.random.Generator | None = None) -> tuple[np.ndarray, np.ndarray]:
    hx, hy, hz = lx / nx, ly / ny, lz / nz
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    coords = np.stack([(i * hx).ravel(), (j * hy).ravel(), (k * hz).ravel()], axis=1).astype(np.float64)
    if jitter > 0.0:
        rng = rng or np.random.default_rng(0)
        interior = ((i > 0) & (i < nx) & (j > 0) & (j < ny) & (k > 0) & (k < nz)).ravel()
        h = np.array([hx, hy, hz])
        d = rng.uniform(-jitter, jitter, size=coords.shape) * h
        coords = np.where(interior[:, None], coords + d, coords)
    ck, cj, ci = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    ci, cj, ck = ci.ravel(), cj.ravel(), ck.ravel()
    kuhn = _kuhn_tets()
    sx, sy = nx + 1, (nx + 1) * (ny + 1)
    conn = np.empty((ci.size, 6, 4), dtype=np.int64)
    for t in range(6):
        for c in range(4):
            ox, oy, oz = kuhn[t, c]
            conn[:, t, c] = (ck + oz) * sy + (cj + oy) * sx + (ci + ox)
    conn = conn.reshape(-1, 4)
    # orient every tet positively (same sign convention as TetVolume)
    p = coords[conn]
    e1, e2, e3 = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]
    vol = np.einsum("ij,ij->i", e1, np.cross(e2, e3))
    neg = vol < 0
    conn[neg, 2], conn[neg, 3] = conn[neg, 3].copy(), conn[neg, 2].copy()
    return coords, conn.astype(np.int32)


def _lognormal(rng: np.random.Generator, n: int, sigma: float) -> np.ndarray:
    return np.exp(sigma * rng.standard_normal(n)).astype(np.float64)


def edge_traction(coords: np.ndarray, nodes: np.ndarray, b: int, traction) -> np.ndarray:
    """Consistent nodal loads of a uniform traction on the polyline ``nodes``:
    each edge adds traction*length/2 to both of its end nodes, edges in order
    (the load the dead code at eqnsys_solid.cpp:558-567 intended)."""
    f = np.zeros(coords.shape[0] * b)
    t = np.asarray(traction, dtype=np.float64)
    nodes = np.asarray(nodes)
    a, c = nodes[:-1], nodes[1:]
    dxy = coords[c] - coords[a]
    L = np.hypot(dxy[:, 0], dxy[:, 1])
    # a node gets at most two edge halves; 0 + x + y is the same in either order
    for d in range(b):
        h = t[d] * L * 0.5
        np.add.at(f, a * b + d, h)
        np.add.at(f, c * b + d, h)
    return f


# --------------------------------------------------------------------------
# the benchmark configurations (seeded)
# --------------------------------------------------------------------------

def poisson2d_square(n: int = 128, seed: int = 1, jitter: float = 0.2, coef_sigma: float = 0.0,
                     tol: float = 1e-8) -> Problem:
    """Unit square, n x n cells, alpha=1, source=1, u=0 on all four edges."""
    rng = np.random.default_rng(seed)
    coords, conn = tri_grid(n, n, 1.0, 1.0, jitter, rng)
    bc = np.zeros(coords.shape[0], dtype=np.int32)
    x, y = coords[:, 0], coords[:, 1]
    bc[(x == 0.0) | (x == 1.0) | (y == 0.0) | (y == 1.0)] = 1
    coef = _lognormal(rng, conn.shape[0], coef_sigma) if coef_sigma > 0 else None
    prm = np.zeros(8); prm[0] = 1.0; prm[1] = 1.0
    return Problem(POISSON2D, coords, conn, prm, bc, coef=coef, tol=tol,
                   name=f"poisson2d_{n}x{n}")


def solid2d_cantilever(nx: int = 1000, ny: int = 500, seed: int = 2, jitter: float = 0.2,
                       coef_sigma: float = 0.5, E: float = 1.0, nu: float = 0.3,
                       traction: float = -1e-3, tol: float = 1e-8) -> Problem:
    """[0, nx/ny] x [0, 1] plane strain, left edge clamped, downward traction on
    the right edge, log-normal per-element E multiplier."""
    rng = np.random.default_rng(seed)
    coords, conn = tri_grid(nx, ny, nx / ny, 1.0, jitter, rng)
    b = 2
    bc = np.zeros(coords.shape[0] * b, dtype=np.int32)
    left = np.nonzero(coords[:, 0] == 0.0)[0]
    bc[left * 2] = 1
    bc[left * 2 + 1] = 1
    right = np.arange(ny + 1) * (nx + 1) + nx
    load = edge_traction(coords, right, b, (0.0, traction))
    coef = _lognormal(rng, conn.shape[0], coef_sigma) if coef_sigma > 0 else None
    lam, myu = lame(E, nu)
    prm = np.zeros(8); prm[0] = lam; prm[1] = myu; prm[2] = 1.0
    return Problem(SOLID2D, coords, conn, prm, bc, coef=coef, load=load, tol=tol,
                   name=f"solid2d_{nx}x{ny}")


def solid3d_cube(n: int = 96, seed: int = 3, coef_sigma: float = 1.0, E: float = 1.0,
                 nu: float = 0.3, gz: float = -1e-3, tol: float = 1e-8, jitter: float = 0.0) -> Problem:
    """Unit cube, n^3 hexes x 6 tets, bottom face clamped, body force gz."""
    rng = np.random.default_rng(seed)
    coords, conn = tet_grid(n, n, n, jitter=jitter, rng=rng)
    b = 3
    bc = np.zeros(coords.shape[0] * b, dtype=np.int32)
    bottom = np.nonzero(coords[:, 2] == 0.0)[0]
    for d in range(3):
        bc[bottom * 3 + d] = 1
    coef = _lognormal(rng, conn.shape[0], coef_sigma) if coef_sigma > 0 else None
    lam, myu = lame(E, nu)
    prm = np.zeros(8); prm[0] = lam; prm[1] = myu; prm[2] = 1.0; prm[5] = gz
    return Problem(SOLID3D, coords, conn, prm, bc, coef=coef, tol=tol, name=f"solid3d_{n}^3")


def poisson3d_cube(n: int = 16, seed: int = 4, coef_sigma: float = 0.0, tol: float = 1e-8) -> Problem:
    rng = np.random.default_rng(seed)
    coords, conn = tet_grid(n, n, n)
    bc = np.zeros(coords.shape[0], dtype=np.int32)
    bc[(coords == 0.0).any(axis=1) | (coords == 1.0).any(axis=1)] = 1
    coef = _lognormal(rng, conn.shape[0], coef_sigma) if coef_sigma > 0 else None
    prm = np.zeros(8); prm[0] = 1.0; prm[1] = 1.0
    return Problem(POISSON3D, coords, conn, prm, bc, coef=coef, tol=tol, name=f"poisson3d_{n}^3")


def diffusion2d_square(n: int = 32, seed: int = 5, rho: float = 1.0, alpha: float = 1.0,
                       source: float = 1.0, gamma: float = 0.5, dt: float = 0.01) -> Problem:
    rng = np.random.default_rng(seed)
    coords, conn = tri_grid(n, n, 1.0, 1.0, 0.2, rng)
    bc = np.zeros(coords.shape[0], dtype=np.int32)
    bc[coords[:, 0] == 0.0] = 1
    u = rng.standard_normal(coords.shape[0]) * 0.1
    v = rng.standard_normal(coords.shape[0]) * 0.1
    prm = np.zeros(8); prm[:5] = (rho, alpha, source, gamma, dt)
    return Problem(DIFFUSION2D, coords, conn, prm, bc, u=u, v=v, name=f"diffusion2d_{n}x{n}")


# --------------------------------------------------------------------------
# request streams of the serving workloads (seeded)
# --------------------------------------------------------------------------

SIDES_2D = ("left", "right", "bottom", "top")
FACES_3D = ("x0", "x1", "y0", "y1", "z0", "z1")


def _side_nodes_2d(nx: int, ny: int, side: str) -> np.ndarray:
    """Node ids along one side of a tri_grid, in order along the side."""
    if side == "left":
        return np.arange(ny + 1) * (nx + 1)
    if side == "right":
        return np.arange(ny + 1) * (nx + 1) + nx
    if side == "bottom":
        return np.arange(nx + 1)
    return ny * (nx + 1) + np.arange(nx + 1)


def rect_problem_2d(kind: int, nnode: int, seed: int, coef_sigma: float = 0.5, jitter: float = 0.2,
                    tol: float = 1e-8) -> Problem:
    """One serving request: a jittered triangulated rectangle of about
    ``nnode`` nodes (aspect ratio log-uniform in [1/4, 4], square cells),
    Poisson (alpha=1, source=1, u=0 on the Dirichlet sides, unit outward flux on
    the load side) or plane-strain elasticity (E=1, nu=0.3, clamped Dirichlet
    sides, traction 1e-3 in a random direction on the load side); 1 to 3 random
    Dirichlet sides, one load side among the rest; log-normal per-element
    multiplier."""
    rng = np.random.default_rng(seed)
    aspect = float(np.exp(rng.uniform(np.log(0.25), np.log(4.0))))
    ny = max(2, int(round(np.sqrt(nnode / aspect))) - 1)
    nx = max(2, int(round(nnode / (ny + 1))) - 1)
    coords, conn = tri_grid(nx, ny, nx / ny, 1.0, jitter, rng)
    b = BLOCK[kind]
    order = rng.permutation(4)
    ndir = int(rng.integers(1, 4))
    dsides = [SIDES_2D[k] for k in order[:ndir]]
    lside = SIDES_2D[order[ndir]]
    bc = np.zeros(coords.shape[0] * b, dtype=np.int32)
    for sd in dsides:
        nodes = _side_nodes_2d(nx, ny, sd)
        for d in range(b):
            bc[nodes * b + d] = 1
    lnodes = _side_nodes_2d(nx, ny, lside)
    coef = _lognormal(rng, conn.shape[0], coef_sigma) if coef_sigma > 0 else None
    prm = np.zeros(8)
    if kind == POISSON2D:
        load = edge_traction(coords, lnodes, 1, (1.0,))
        prm[0] = 1.0
        prm[1] = 1.0
    elif kind == SOLID2D:
        ang = rng.uniform(0.0, 2.0 * np.pi)
        load = edge_traction(coords, lnodes, 2, (1e-3 * np.cos(ang), 1e-3 * np.sin(ang)))
        lam, myu = lame(1.0, 0.3)
        prm[0] = lam
        prm[1] = myu
        prm[2] = 1.0
    else:
        raise ValueError("2D serving requests are Poisson or plane-strain elasticity")
    load[bc != 0] = 0.0
    return Problem(kind, coords, conn, prm, bc, coef=coef, load=load, tol=tol,
                   name=f"{KIND_NAMES[kind]}_{nx}x{ny}")


def box_problem_3d(kind: int, nx: int, ny: int, nz: int, seed: int, coef_sigma: float = 1.0,
                   tol: float = 1e-8) -> Problem:
    """One 3D serving request: an nx x ny x nz hex grid of unit cells split
    into Kuhn tetrahedra; Poisson (alpha=1, source=1) or elasticity (E=1,
    nu=0.3, body force -1e-3 along z); 1 to 3 random Dirichlet faces (u=0 /
    clamped); log-normal per-element multiplier."""
    rng = np.random.default_rng(seed)
    coords, conn = tet_grid(nx, ny, nz, float(nx), float(ny), float(nz))
    b = BLOCK[kind]
    order = rng.permutation(6)
    ndir = int(rng.integers(1, 4))
    ext = (nx, ny, nz)
    bcn = np.zeros(coords.shape[0], dtype=bool)
    for f in order[:ndir]:
        axis, hi = divmod(int(f), 2)
        bcn |= coords[:, axis] == (float(ext[axis]) if hi else 0.0)
    bc = np.repeat(bcn.astype(np.int32), b)
    coef = _lognormal(rng, conn.shape[0], coef_sigma) if coef_sigma > 0 else None
    prm = np.zeros(8)
    if kind == POISSON3D:
        prm[0] = 1.0
        prm[1] = 1.0
    elif kind == SOLID3D:
        lam, myu = lame(1.0, 0.3)
        prm[0] = lam
        prm[1] = myu
        prm[2] = 1.0
        prm[5] = -1e-3
    else:
        raise ValueError("3D serving requests are Poisson or elasticity")
    return Problem(kind, coords, conn, prm, bc, coef=coef, tol=tol, name=f"{KIND_NAMES[kind]}_{nx}x{ny}x{nz}")


@dataclasses.dataclass
class StreamItem:
    arrival: float      # seconds after the stream starts
    kind: int
    size: tuple         # 2D: (target nodes,); 3D: (nx, ny, nz)
    seed: int

    def problem(self) -> Problem:
        if len(self.size) == 1:
            return rect_problem_2d(self.kind, self.size[0], self.seed)
        return box_problem_3d(self.kind, *self.size, seed=self.seed)


def serve_stream_2d(nreq: int = 2000, seed: int = 4, rate: float = 200.0, nmin: int = 2000,
                    nmax: int = 400000) -> list[StreamItem]:
    """Poisson arrivals at ``rate`` requests/s; 50/50 Poisson and plane-strain
    elasticity; node counts log-uniform in [nmin, nmax]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, nreq))
    sizes = np.exp(rng.uniform(np.log(nmin), np.log(nmax), nreq)).astype(int)
    kinds = np.where(rng.random(nreq) < 0.5, POISSON2D, SOLID2D)
    seeds = rng.integers(0, 2**31 - 1, nreq)
    return [StreamItem(float(t[i]), int(kinds[i]), (int(sizes[i]),), int(seeds[i])) for i in range(nreq)]


def serve_stream_3d(nreq: int = 500, seed: int = 5, rate: float = 50.0, emin: int = 16,
                    emax: int = 80) -> list[StreamItem]:
    """Poisson arrivals; 50/50 3D Poisson and 3D elasticity; hex-grid edge
    counts per axis uniform in [emin, emax]."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, nreq))
    ext = rng.integers(emin, emax + 1, size=(nreq, 3))
    kinds = np.where(rng.random(nreq) < 0.5, POISSON3D, SOLID3D)
    seeds = rng.integers(0, 2**31 - 1, nreq)
    return [StreamItem(float(t[i]), int(kinds[i]), tuple(int(v) for v in ext[i]), int(seeds[i]))
            for i in range(nreq)]


# --------------------------------------------------------------------------
# problem file (read by oracle/ref_harness.cpp)
# --------------------------------------------------------------------------

PROBLEM_MAGIC = 0x44464731
RESULT_MAGIC = 0x44464733


def write_problem(p: Problem, path: str) -> None:
    b, ndim = p.b, NDIM[p.kind]
    with open(path, "wb") as f:
        f.write(struct.pack("<7i", PROBLEM_MAGIC, p.kind, p.nnode, ndim, p.nelem, p.conn.shape[1], b))
        f.write(np.ascontiguousarray(p.coords, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(p.conn, dtype="<i4").tobytes())
        for arr, dt in ((p.coef, "<f8"),):
            f.write(struct.pack("<i", 0 if arr is None else 1))
            if arr is not None:
                f.write(np.ascontiguousarray(arr, dtype=dt).tobytes())
        f.write(np.ascontiguousarray(p.params, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(p.bcflag, dtype="<i4").tobytes())
        for arr in (p.load, p.u, p.v):
            f.write(struct.pack("<i", 0 if arr is None else 1))
            if arr is not None:
                f.write(np.ascontiguousarray(arr, dtype="<f8").tobytes())
        f.write(struct.pack("<di", p.tol, p.maxit))


def read_result(path: str) -> dict:
    raw = open(path, "rb").read()
    off = 0

    def take(fmt_or_dtype, count=None):
        nonlocal off
        if count is None:
            v = struct.unpack_from(fmt_or_dtype, raw, off)
            off += struct.calcsize(fmt_or_dtype)
            return v
        a = np.frombuffer(raw, dtype=fmt_or_dtype, count=count, offset=off).copy()
        off += a.nbytes
        return a

    magic, n, b, nnz = take("<4i")
    assert magic == RESULT_MAGIC
    bs = b * b
    out = dict(n=n, b=b, nnz=nnz)
    out["rowptr"] = take("<i4", n + 1)
    out["colind"] = take("<i4", nnz)
    out["diag"] = take("<f8", n * bs)
    out["offd"] = take("<f8", nnz * bs)
    out["rhs"] = take("<f8", n * b)
    (out["norm_res"],) = take("<d")
    out["ilu_ok"], out["prec_ok"] = take("<2i")
    out["fill_level"], nnz_f = take("<2i")
    out["rowptr_f"] = take("<i4", n + 1)
    out["colind_f"] = take("<i4", nnz_f)
    out["fdiag"] = take("<f8", n * bs)
    out["foffd"] = take("<f8", nnz_f * bs)
    out["converged"], out["iter"] = take("<2i")
    (out["conv"],) = take("<d")
    out["x"] = take("<f8", n * b)
    return out


# ------------------------------------------------------------ GiD mesh files

def read_gid_msh(path: str):
    """Nodes and elements of a GiD ".msh" file through the library's reader
    (dfg_mesh_read_gid; no device needed): (coords (nnode, ndim), conn
    (nelem, nnoel) 0-based), triangles in 2D or tetrahedra in 3D."""
    import ctypes
    from . import capi
    L = capi.lib()
    nd, nk, nn, ne = (ctypes.c_int() for _ in range(4))
    st = L.dfg_mesh_read_gid(path.encode(), ctypes.byref(nd), ctypes.byref(nk), ctypes.byref(nn),
                             ctypes.byref(ne), None, None)
    if st != capi.DFG_OK:
        raise capi.DfgError(st, "dfg_mesh_read_gid", L.dfg_last_error(None).decode(errors="replace"))
    coords = np.zeros((nn.value, nd.value))
    conn = np.zeros((ne.value, nk.value), dtype=np.int32)
    st = L.dfg_mesh_read_gid(path.encode(), ctypes.byref(nd), ctypes.byref(nk), ctypes.byref(nn), ctypes.byref(ne),
                             ctypes.c_void_p(coords.ctypes.data), ctypes.c_void_p(conn.ctypes.data))
    if st != capi.DFG_OK:
        raise capi.DfgError(st, "dfg_mesh_read_gid", L.dfg_last_error(None).decode(errors="replace"))
    return coords, conn


def write_gid_msh(path: str, coords: np.ndarray, conn: np.ndarray) -> None:
    """Writes a GiD ".msh" file in the layout of the reference's input meshes
    (three coordinates per node, 17 significant digits so that reading it
    back gives the same doubles)."""
    nnoel = conn.shape[1]
    etype = {3: "Triangle", 4: "Tetrahedra"}[nnoel]
    with open(path, "w") as f:
        f.write(f"MESH    dimension 3 ElemType {etype}  Nnode {nnoel}\nCoordinates\n")
        for i, c in enumerate(coords):
            xyz = list(c) + [0.0] * (3 - len(c))
            f.write(f"{i + 1:6d} {xyz[0]:.17g} {xyz[1]:.17g} {xyz[2]:.17g}\n")
        f.write("end coordinates\n\nElements\n")
        for e, v in enumerate(conn):
            f.write(f"{e + 1:6d} " + " ".join(str(int(x) + 1) for x in v) + "\n")
        f.write("end elements\n")


def boundary_nodes(conn: np.ndarray) -> np.ndarray:
    """Nodes on the boundary of a triangle or tetrahedron mesh: those of the
    edges (faces) that belong to one element only."""
    k = conn.shape[1]
    faces = np.sort(np.concatenate([np.delete(conn, j, axis=1) for j in range(k)]), axis=1)
    uniq, counts = np.unique(faces, axis=0, return_counts=True)
    return np.unique(uniq[counts == 1].ravel())


def mesh_problem(kind: int, coords: np.ndarray, conn: np.ndarray, seed: int = 0, coef_sigma: float = 0.0,
                 tol: float = 1e-8, name: str = "mesh") -> Problem:
    """A load case on a given mesh: Poisson kinds with alpha = source = 1 and
    u = 0 on every boundary node; solid kinds clamped on the boundary nodes of
    smallest x, under gravity -1e-3 along the last axis (E = 1, nu = 0.3)."""
    rng = np.random.default_rng(seed)
    coords = np.ascontiguousarray(coords, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int32)
    b = BLOCK[kind]
    bnd = boundary_nodes(conn)
    bc = np.zeros(coords.shape[0] * b, dtype=np.int32)
    prm = np.zeros(8)
    if kind in (POISSON2D, POISSON3D):
        bc[bnd] = 1
        prm[0] = 1.0
        prm[1] = 1.0
    elif kind in (SOLID2D, SOLID3D):
        xmin = coords[:, 0].min()
        clamp = bnd[np.abs(coords[bnd, 0] - xmin) <= 1e-9 * max(1.0, abs(xmin))]
        for d in range(b):
            bc[clamp * b + d] = 1
        lam, myu = lame(1.0, 0.3)
        prm[0] = lam
        prm[1] = myu
        prm[2] = 1.0
        prm[2 + b] = -1e-3  # g_y in 2D (params[4]), g_z in 3D (params[5])
    else:
        raise ValueError("mesh_problem covers the Poisson and solid kinds")
    coef = _lognormal(rng, conn.shape[0], coef_sigma) if coef_sigma > 0 else None
    return Problem(kind, coords, conn, prm, bc, coef=coef, tol=tol, name=name)


def delaunay_mesh(npoints: int, dim: int, seed: int = 0):
    """An unstructured P1 mesh: the Delaunay triangulation (dim 2) or
    tetrahedralisation (dim 3) of seeded random points in the unit square or
    cube plus its corners, elements oriented positively, nodes in the random
    order they were drawn (irregular valences and bandwidth).  Needs scipy."""
    from scipy.spatial import Delaunay
    rng = np.random.default_rng(seed)
    corners = np.array(list(itertools.product([0.0, 1.0], repeat=dim)))
    pts = np.vstack([corners, rng.random((npoints, dim))])
    conn = Delaunay(pts).simplices.astype(np.int32)
    # orientation: positive area / volume
    v = pts[conn[:, 1:]] - pts[conn[:, :1]]
    det = np.linalg.det(v)
    flip = det < 0
    conn[flip, 0], conn[flip, 1] = conn[flip, 1].copy(), conn[flip, 0].copy()
    keep = np.abs(det) > 1e-12  # drop slivers of zero measure
    return pts, np.ascontiguousarray(conn[keep])
