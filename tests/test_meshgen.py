"""Synthetic workloads: sizes of the benchmark configurations (node, element
and off-diagonal block counts from the grid topology) and basic invariants."""
import numpy as np
import pytest

from delfem_gb300 import meshgen as mg


def tri_counts(nx, ny):
    n = (nx + 1) * (ny + 1)
    edges = nx * (ny + 1) + ny * (nx + 1) + nx * ny  # horizontal, vertical, diagonal
    return n, 2 * edges, 2 * nx * ny


def test_config_sizes_2d():
    for nx, ny in ((128, 128), (1000, 500)):
        n, z, e = tri_counts(nx, ny)
        if nx == 128:
            assert (n, z, e) == (16641, 98816, 32768)
        else:
            assert (n, z, e) == (501501, 3003000, 1000000)


def test_pattern_counts_match_topology(oracle_lib):
    coords, conn = mg.tri_grid(7, 5)
    rowptr, colind = oracle_lib.pattern(coords.shape[0], conn)
    n, z, e = tri_counts(7, 5)
    assert rowptr[-1] == z and conn.shape[0] == e and coords.shape[0] == n


def test_tet_grid_counts_and_orientation(oracle_lib):
    coords, conn = mg.tet_grid(4, 3, 2)
    assert coords.shape[0] == 5 * 4 * 3 and conn.shape[0] == 6 * 4 * 3 * 2
    p = coords[conn]
    vol = np.einsum("ij,ij->i", p[:, 1] - p[:, 0], np.cross(p[:, 2] - p[:, 0], p[:, 3] - p[:, 0]))
    assert (vol > 0).all()
    assert np.isclose(vol.sum() / 6.0, 1.0)
    # 96^3 configuration: 912,673 nodes and 12,552,768 off-diagonal blocks (edges of the Kuhn grid x 2)
    n96 = 97 ** 3
    edges = 3 * 96 * 97 * 97 + 3 * 96 * 96 * 97 + 96 ** 3
    assert n96 == 912673 and 2 * edges == 12552768
    rowptr, _ = oracle_lib.pattern(coords.shape[0], conn)
    nx, ny, nz = 4, 3, 2
    e3 = (nx * (ny + 1) * (nz + 1) + ny * (nx + 1) * (nz + 1) + nz * (nx + 1) * (ny + 1)
          + nx * ny * (nz + 1) + nx * nz * (ny + 1) + ny * nz * (nx + 1) + nx * ny * nz)
    assert rowptr[-1] == 2 * e3


def test_seeded_and_jittered():
    a = mg.solid2d_cantilever(20, 10, seed=5)
    b = mg.solid2d_cantilever(20, 10, seed=5)
    assert np.array_equal(a.coords, b.coords) and np.array_equal(a.coef, b.coef)
    h = 1.0 / 10
    i = np.arange(a.nnode) % 21
    j = np.arange(a.nnode) // 21
    interior = (i > 0) & (i < 20) & (j > 0) & (j < 10)
    dx = a.coords[:, 0] - i * h
    assert np.abs(dx[interior]).max() <= 0.2 * h + 1e-15
    assert np.all(dx[~interior] == 0)


def test_traction_is_consistent():
    p = mg.solid2d_cantilever(10, 5, traction=-1e-3)
    f = p.load.reshape(-1, 2)
    assert np.isclose(f[:, 1].sum(), -1e-3 * 1.0)
    assert np.all(f[:, 0] == 0)


@pytest.mark.parametrize("sigma", [0.5, 1.0])
def test_lognormal_coefficients(sigma):
    p = mg.solid3d_cube(6, coef_sigma=sigma)
    lg = np.log(p.coef)
    assert abs(lg.std() - sigma) < 0.05 and abs(lg.mean()) < 0.05


def test_serving_streams_match_their_distributions():
    from delfem_gb300 import meshgen as mg
    st = mg.serve_stream_2d(rate=50.0)
    assert len(st) == 2000
    t = np.array([it.arrival for it in st])
    assert np.all(np.diff(t) > 0) and 36 < t[-1] < 44           # Poisson arrivals at 50/s
    sizes = np.array([it.size[0] for it in st])
    assert sizes.min() >= 2000 and sizes.max() <= 400000
    kinds = np.array([it.kind for it in st])
    assert set(kinds) == {mg.POISSON2D, mg.SOLID2D} and 0.45 < np.mean(kinds == mg.POISSON2D) < 0.55
    again = mg.serve_stream_2d(rate=50.0)
    assert [(a.seed, a.size, a.kind) for a in again[:50]] == [(b.seed, b.size, b.kind) for b in st[:50]]
    s3 = mg.serve_stream_3d()
    assert len(s3) == 500 and all(16 <= e <= 80 for it in s3 for e in it.size)


def test_serving_requests_are_well_posed():
    from delfem_gb300 import meshgen as mg
    for it in mg.serve_stream_2d(nreq=12, seed=3, nmin=300, nmax=5000):
        p = it.problem()
        assert abs(p.nnode - it.size[0]) <= 0.25 * it.size[0] + 20
        assert p.bcflag.any()                                    # at least one Dirichlet side
        assert p.load is not None and not np.any(p.load[p.bcflag != 0])
        assert p.coef is not None and np.all(p.coef > 0)
        e1 = p.coords[p.conn[:, 1]] - p.coords[p.conn[:, 0]]
        e2 = p.coords[p.conn[:, 2]] - p.coords[p.conn[:, 0]]
        assert np.all(e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0] > 0)   # counter-clockwise, non-degenerate
    for it in mg.serve_stream_3d(nreq=3, seed=4, emin=3, emax=5):
        p = it.problem()
        assert p.bcflag.any() and p.nnode == np.prod([e + 1 for e in it.size])
