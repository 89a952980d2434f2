"""Known answers for the oracle and the reference, beside the golden
fixtures' bit-for-bit agreement.
* Patch tests: the element matrices of one element against closed forms
  (P1 Poisson on a triangle and a tetrahedron) and against the rigid-body
  null space (linear elasticity in 2D and 3D).
* tests/golden/known/: fixtures the reference itself produced for problems
  with closed-form answers. The oracle must reproduce every step bit for bit.
  A 2 x 2 Poisson grid's matrix, right-hand side, factor and solution equal
  their hand-computed values. Linear fields set on the boundary are
  reproduced exactly in the interior (P1 elements contain them)."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN_DIR, bits, load_golden

KNOWN = sorted(glob.glob(os.path.join(GOLDEN_DIR, "known", "*.npz")))


def _dense(oracle_lib, p):
    """The element assembly of p (before Dirichlet) as a dense matrix and the
    residual vector."""
    rp, ci = oracle_lib.pattern(p.nnode, p.conn)
    diag, offd, res = oracle_lib.assemble(p, rp, ci)
    n, b = p.nnode, p.b
    bs = b * b
    K = np.zeros((n * b, n * b))
    for i in range(n):
        K[i * b:(i + 1) * b, i * b:(i + 1) * b] = diag[i * bs:(i + 1) * bs].reshape(b, b)
        for c in range(rp[i], rp[i + 1]):
            j = ci[c]
            K[i * b:(i + 1) * b, j * b:(j + 1) * b] = offd[c * bs:(c + 1) * bs].reshape(b, b)
    return K, res


def _one_element(kind, coords, prm):
    from delfem_gb300 import meshgen as mg
    coords = np.asarray(coords, dtype=np.float64)
    conn = np.arange(coords.shape[0], dtype=np.int32)[None, :]
    b = mg.BLOCK[kind]
    return mg.Problem(kind, coords, conn, np.asarray(prm, dtype=np.float64),
                      np.zeros(coords.shape[0] * b, dtype=np.int32))


def test_poisson_triangle_closed_form(oracle_lib):
    """Unit right triangle, alpha = 2, source = 3: K = alpha * area * G G^T
    with gradients G = (-1,-1), (1,0), (0,1) and area 1/2; residual
    source * area / 3 per node (eqn_poisson.cpp:49-125)."""
    from delfem_gb300 import meshgen as mg
    p = _one_element(mg.POISSON2D, [[0, 0], [1, 0], [0, 1]], [2.0, 3.0, 0, 0, 0, 0, 0, 0])
    K, res = _dense(oracle_lib, p)
    G = np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0]])
    np.testing.assert_allclose(K, 2.0 * 0.5 * G @ G.T, rtol=0, atol=1e-15)
    np.testing.assert_allclose(res, np.full(3, 3.0 * 0.5 / 3.0), rtol=1e-15)


def test_poisson_tetrahedron_closed_form(oracle_lib):
    """Unit corner tetrahedron, alpha = 1.5, source = 2: K = alpha * vol * G G^T
    with gradients (-1,-1,-1), e1, e2, e3 and vol = 1/6; residual
    source * vol / 4 per node.  The reference's volume uses the truncated
    literal 0.1666666666666 for 1/6 (ker_emat_tet.h:32-39), which moves K
    and the residual by about 4e-13 relative."""
    from delfem_gb300 import meshgen as mg
    p = _one_element(mg.POISSON3D, [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], [1.5, 2.0, 0, 0, 0, 0, 0, 0])
    K, res = _dense(oracle_lib, p)
    G = np.array([[-1.0, -1.0, -1.0], [1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0]])
    np.testing.assert_allclose(K, 1.5 / 6.0 * G @ G.T, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(res, np.full(4, 2.0 / 6.0 / 4.0), rtol=1e-12)
    assert not np.array_equal(res, np.full(4, 2.0 / 6.0 / 4.0))  # the truncated literal shows


def _rigid_modes(coords):
    """Translations and infinitesimal rotations of the nodes (2D: 3, 3D: 6)."""
    n, d = coords.shape
    modes = []
    for a in range(d):
        t = np.zeros((n, d))
        t[:, a] = 1.0
        modes.append(t.ravel())
    pairs = [(0, 1)] if d == 2 else [(0, 1), (1, 2), (0, 2)]
    for a, c in pairs:
        r = np.zeros((n, d))
        r[:, a], r[:, c] = -coords[:, c], coords[:, a]
        modes.append(r.ravel())
    return np.array(modes).T


@pytest.mark.parametrize("dim", [2, 3])
def test_elasticity_element_null_space(oracle_lib, dim):
    """A skewed linear-elastic element (eqn_linear_solid2d.cpp:505-598,
    eqn_linear_solid3d.cpp:241-334): symmetric, positive semi-definite, its
    null space exactly the rigid-body motions (3 in 2D, 6 in 3D), and no
    residual without body force."""
    from delfem_gb300 import meshgen as mg
    E, nu = 2.5, 0.3
    lam, myu = E * nu / ((1 + nu) * (1 - 2 * nu)), E / (2 * (1 + nu))
    if dim == 2:
        co = [[0.1, 0.0], [1.3, 0.2], [0.4, 0.9]]
        p = _one_element(mg.SOLID2D, co, [lam, myu, 1.0, 0.0, 0.0, 0, 0, 0])
    else:
        co = [[0.0, 0.1, 0.0], [1.1, 0.0, 0.2], [0.2, 0.9, 0.1], [0.3, 0.2, 1.2]]
        p = _one_element(mg.SOLID3D, co, [lam, myu, 1.0, 0.0, 0.0, 0.0, 0, 0])
    K, res = _dense(oracle_lib, p)
    np.testing.assert_allclose(K, K.T, rtol=0, atol=1e-14 * np.abs(K).max())
    w = np.linalg.eigvalsh(0.5 * (K + K.T))
    nrb = 3 if dim == 2 else 6
    scale = np.abs(w).max()
    assert np.all(np.abs(w[:nrb]) < 1e-12 * scale) and np.all(w[nrb:] > 1e-6 * scale)
    R = _rigid_modes(np.asarray(co))
    assert np.abs(K @ R).max() < 1e-13 * scale
    assert not np.any(res)


def test_known_fixtures_present():
    names = [os.path.basename(f) for f in KNOWN]
    assert len(names) == 4 and names[0].startswith("00_poisson2d_2x2")


@pytest.mark.parametrize("path", KNOWN, ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_oracle_matches_reference_on_known(path, oracle_lib):
    p, ref = load_golden(path)
    out = oracle_lib.solve(p)
    assert np.array_equal(out["rowptr"], ref["rowptr"]) and np.array_equal(out["colind"], ref["colind"])
    for k in ("diag", "offd", "rhs", "fdiag", "foffd", "x"):
        assert np.array_equal(bits(out[k]), bits(ref[k])), k
    assert out["iter"] == int(ref["iter"]) and out["conv"] == float(ref["conv"])


def test_two_by_two_grid_by_hand(oracle_lib):
    """Every step of the 2 x 2 grid (h = 1/2, alpha = source = 1), from the
    reference's run: before Dirichlet the centre row is 4 on the diagonal, -1
    to the four axis neighbours and 0 to the two along the split diagonal
    (cotangents of 45 and 90 degrees); after it the centre row keeps only 4
    and the right-hand side only source * h^2 = 0.25 at the centre; the
    factor's pivot is 1/4; PCG converges at iteration 0 with u = 1/16."""
    p, ref = load_golden(KNOWN[0])
    c = 4  # the centre node
    rp, ci = oracle_lib.pattern(p.nnode, p.conn)
    diag, offd, _ = oracle_lib.assemble(p, rp, ci)
    cols = ci[rp[c]:rp[c + 1]]
    vals = dict(zip(cols.tolist(), offd[rp[c]:rp[c + 1]].tolist()))
    assert diag[c] == 4.0
    assert vals == {0: 0.0, 1: -1.0, 3: -1.0, 5: -1.0, 7: -1.0, 8: 0.0}
    rp_r = ref["rowptr"]
    assert ref["diag"][c] == 4.0 and not np.any(ref["offd"][rp_r[c]:rp_r[c + 1]])
    rhs = ref["rhs"]
    assert rhs[c] == pytest.approx(0.25, rel=1e-15) and not np.any(np.delete(rhs, c))
    assert ref["fdiag"][c] == 0.25
    assert int(ref["iter"]) == 0 and bool(ref["converged"])
    assert ref["x"][c] == pytest.approx(1.0 / 16.0, rel=1e-15) and not np.any(np.delete(ref["x"], c))


@pytest.mark.parametrize("path", KNOWN[1:], ids=lambda p: p.rsplit("/", 1)[-1][:-4])
def test_linear_field_reproduced(path, oracle_lib):
    """Dirichlet lifting of a linear field: field + update equals the field
    at every node, in the reference's run and in the oracle's."""
    p, ref = load_golden(path)
    # the field on the boundary and, as the fixture stores it, zero inside:
    # recover the linear field from the boundary values by least squares
    bnd = p.bcflag.reshape(p.nnode, p.b)[:, 0] == 1
    A = np.hstack([np.ones((p.nnode, 1)), p.coords])
    coef, *_ = np.linalg.lstsq(A[bnd], p.u.reshape(p.nnode, p.b)[bnd], rcond=None)
    g = (A @ coef).ravel()
    assert np.abs(p.u.reshape(p.nnode, p.b)[bnd] - (A @ coef)[bnd]).max() < 1e-13
    for x in (ref["x"], oracle_lib.solve(p)["x"]):
        np.testing.assert_allclose(p.u + x, g, rtol=0, atol=1e-10 * np.abs(g).max())
