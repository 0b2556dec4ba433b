"""Known answers and properties of the oracle (CPU only)."""
import numpy as np
import pytest
import scipy.sparse as sp

from arcanefem_gb300 import meshgen
from oracle import oracle as O


def test_element_known_answers():
    # right triangle (0,0) (1,0) (0,1): K = 1/2 [[2,-1,-1],[-1,1,0],[-1,0,1]]
    c = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], float)
    K = np.array([O.elem_vec(O.POISSON_TRI3, c, [0, 1, 2], i) for i in range(3)])
    np.testing.assert_allclose(K, 0.5 * np.array([[2, -1, -1], [-1, 1, 0], [-1, 0, 1]]), atol=1e-15)
    Kt = np.array([O.elem_vec(O.TESTLAB_TRI3, c, [0, 1, 2], i) for i in range(3)])
    np.testing.assert_allclose(Kt, K, atol=1e-15)
    # unit tetrahedron: K = 1/6 [[3,-1,-1,-1],[-1,1,0,0],[-1,0,1,0],[-1,0,0,1]]
    c = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    ref = np.array([[3, -1, -1, -1], [-1, 1, 0, 0], [-1, 0, 1, 0], [-1, 0, 0, 1]]) / 6
    K = np.array([O.elem_vec(O.POISSON_TET4, c, [0, 1, 2, 3], i) for i in range(4)])
    np.testing.assert_allclose(K, ref, atol=1e-15)
    Kt = np.array([O.elem_vec(O.TESTLAB_TET4, c, [0, 1, 2, 3], i) for i in range(4)])
    np.testing.assert_allclose(Kt, ref, atol=1e-15)


def test_elasticity_element_rigid_modes_and_symmetry():
    rng = np.random.default_rng(0)
    c = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float) + 0.1 * rng.standard_normal((4, 3))
    lam, mu = 2.0, 0.7
    K = np.vstack([O.elem_vec(O.ELASTICITY_TET4, c, [0, 1, 2, 3], i, lam, mu) for i in range(4)])
    assert np.abs(K - K.T).max() < 1e-12 * np.abs(K).max()
    for t in np.eye(3):                       # translations
        assert np.abs(K @ np.tile(t, 4)).max() < 1e-12 * np.abs(K).max()
    rot = np.cross(np.array([0.3, -0.2, 0.5]), c).ravel()   # infinitesimal rotation
    assert np.abs(K @ rot).max() < 1e-11 * np.abs(K).max()


def _csr(vals, cols, rp, n):
    return sp.csr_matrix((vals, cols, rp), shape=(n, n))


def test_nodewise_assembly_properties():
    for m, kind in ((meshgen.unit_square_tri(6, seed=2), O.POISSON_TRI3),
                    (meshgen.unit_cube_tet(3, seed=2), O.POISSON_TET4)):
        ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
        rp, cols = O.sparsity(m.nb_node, m.cells)
        assert rp[-1] == meshgen.nnz_formula(m)
        v = O.assemble(kind, m.coords, m.cells, ptr, nc, rp, cols)
        A = _csr(v, cols, rp, m.nb_node)
        assert abs(A - A.T).max() < 1e-14 * abs(A).max()
        assert np.abs(A @ np.ones(m.nb_node)).max() < 1e-13 * abs(A).max()
        # self-last order holds the same set of columns with the diagonal last
        rp2, cols2 = O.sparsity(m.nb_node, m.cells, self_last=True)
        assert np.array_equal(rp, rp2)
        for i in range(m.nb_node):
            row = cols2[rp2[i]:rp2[i + 1]]
            assert row[-1] == i and np.array_equal(np.sort(row), cols[rp[i]:rp[i + 1]])
        v2 = O.assemble(kind, m.coords, m.cells, ptr, nc, rp2, cols2)
        A2 = _csr(v2, cols2, rp2, m.nb_node)
        assert abs(A - A2).max() == 0.0


def test_elasticity_layouts_agree():
    m = meshgen.unit_cube_tet(2, seed=5)
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    rp, cols = O.sparsity(m.nb_node, m.cells)
    lam, mu = 3.0, 1.0
    vr = O.assemble(O.ELASTICITY_TET4, m.coords, m.cells, ptr, nc, rp, cols, per_block_layout=False, lam=lam, mu=mu)
    vb = O.assemble(O.ELASTICITY_TET4, m.coords, m.cells, ptr, nc, rp, cols, per_block_layout=True, lam=lam, mu=mu)
    for r in range(m.nb_node):
        L = rp[r + 1] - rp[r]
        for x in range(L):
            for i in range(3):
                for j in range(3):
                    a = vr[rp[r] * 9 + 3 * (x + i * L) + j]
                    b = vb[(rp[r] + x) * 9 + 3 * i + j]
                    assert a == b


def _reference_transform(rp, cols, vals, rhs, fi, fv, ei, ev):
    """Direct numpy statement of CsrDoFLinearSystemImpl (incl. the column_index > 0 test)."""
    n = rp.size - 1
    vals, rhs = vals.copy(), rhs.copy()
    has_rc = (ei == 2).any()
    saved = {}
    if has_rc:
        for i in range(n):
            for k in range(rp[i], rp[i + 1]):
                j = cols[k]
                if ei[i] == 2 or ei[j] == 2:
                    saved[(i, j)] = vals[k]
    for i in range(n):
        if ei[i] == 1:
            for k in range(rp[i], rp[i + 1]):
                vals[k] = 1.0 if cols[k] == i else 0.0
    if has_rc:
        for i in range(n):
            for k in range(rp[i], rp[i + 1]):
                j = cols[k]
                if j > 0 and (ei[i] in (1, 2) or ei[j] in (1, 2)):
                    vals[k] = 1.0 if j == i else 0.0
    for i in range(n):
        if fi[i]:
            for k in range(rp[i], rp[i + 1]):
                if cols[k] == i:
                    vals[k] = fv[i]
    for (i, j), a in sorted(saved.items()):
        if i != j and ei[i] == 2:
            rhs[j] = rhs[j] - a * ev[i]
    for i in range(n):
        if ei[i] in (1, 2):
            rhs[i] = ev[i]
    return vals, rhs


def test_dirichlet_transformations_match_reference_semantics():
    rng = np.random.default_rng(1)
    m = meshgen.unit_square_tri(4, seed=1)
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    rp, cols = O.sparsity(m.nb_node, m.cells)
    v = O.assemble(O.POISSON_TRI3, m.coords, m.cells, ptr, nc, rp, cols)
    n = m.nb_node
    rhs = rng.standard_normal(n)
    fi, fv = np.zeros(n, np.uint8), np.zeros(n)
    ei, ev = np.zeros(n, np.uint8), np.zeros(n)
    # node 0 row-column eliminated: exercises the column_index > 0 quirk
    O.dirichlet_elimination(np.array([0, 3, 7]), 1, 0, 0.25, 2, ei, ev)
    O.dirichlet_elimination(np.array([12, 13]), 1, 0, -1.5, 1, ei, ev)
    O.dirichlet_penalty(np.array([20, 21]), 1, 0, 2.0, 1e30, fi, fv, rhs)
    ev_vals, ev_rhs = _reference_transform(rp, cols, v, rhs, fi, fv, ei, ev)
    vv, rr = v.copy(), rhs.copy()
    O.apply_transformations(rp, cols, vv, rr, fi, fv, ei, ev)
    assert np.array_equal(vv, ev_vals)
    assert np.array_equal(rr, ev_rhs)
    # the quirk: the diagonal of row 0 is not reset to 1
    k0 = rp[0] + list(cols[rp[0]:rp[1]]).index(0)
    assert vv[k0] == v[k0] and v[k0] != 1.0


@pytest.mark.parametrize("dim", [2, 3])
def test_boundary_face_terms_integrate_the_boundary(dim):
    """Neumann / traction terms of the oracle: a scalar flux integrates to
    g x |boundary|, a constant vector's normal flux to 0 (divergence theorem),
    a traction to g x |boundary| per component; the face orientation flags
    are honoured (a flipped face with its flag flipped gives the same sum)."""
    from arcanefem_gb300 import meshgen
    m = meshgen.unit_square_tri(6, seed=3) if dim == 2 else meshgen.unit_cube_tet(4, seed=3)
    f, out = meshgen.boundary_faces(m, seed=5)
    size = 4.0 if dim == 2 else 6.0
    r = O.rhs_boundary_faces(dim, m.coords, f, out, O.FACE_SCALAR, [2.5], 1, np.zeros(m.nb_node))
    assert abs(r.sum() - 2.5 * size) < 1e-12
    g = [1.0, -2.0, 0.5][:dim]
    r = O.rhs_boundary_faces(dim, m.coords, f, out, O.FACE_NORMAL, g, 1, np.zeros(m.nb_node))
    assert abs(r.sum()) < 1e-12
    # outward normal flux of the position field x integrates to dim x volume: use g = e_x on the x = 1 face only
    r = O.rhs_boundary_faces(dim, m.coords, f, out, O.FACE_VECTOR, g, dim, np.zeros(m.nb_node * dim))
    assert np.allclose(r.reshape(-1, dim).sum(0), np.array(g) * size, atol=1e-12)
    # flipping a face's first two nodes together with its flag leaves the normal flux unchanged
    f2, out2 = f.copy(), out.copy()
    f2[:, [0, 1]] = f2[:, [1, 0]]
    out2 = 1 - out2
    ra = O.rhs_boundary_faces(dim, m.coords, f, out, O.FACE_NORMAL, g, 1, np.zeros(m.nb_node))
    rb = O.rhs_boundary_faces(dim, m.coords, f2, out2, O.FACE_NORMAL, g, 1, np.zeros(m.nb_node))
    assert np.allclose(ra, rb, atol=1e-14)
    # the x = 1 face carries flux +|face| for g = e_x
    on = np.all(np.isclose(m.coords[f, 0], 1.0), axis=1)
    r = O.rhs_boundary_faces(dim, m.coords, f[on], out[on], O.FACE_NORMAL, [1.0, 0.0, 0.0][:dim], 1,
                             np.zeros(m.nb_node))
    assert abs(r.sum() - 1.0) < 1e-12


@pytest.mark.parametrize("dim", [2, 3])
def test_q1_source_integrates_the_domain(dim):
    """The Quad4 / Hexa8 constant source sums to qdot x |domain| (2x2(x2) Gauss
    points integrate the shape functions exactly)."""
    from arcanefem_gb300 import meshgen
    m = meshgen.unit_square_quad(9, seed=2) if dim == 2 else meshgen.unit_cube_hex(4, seed=2)
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    r = O.rhs_constant_source_q1(dim, m.coords, m.cells, ptr, nc, 2.5)
    assert abs(r.sum() - 2.5) < 1e-12


def test_cpu_baselines_compute_the_same_matrix():
    """The timed CPU baselines are the same computation: the DOK assembly
    (ordered map, zeros skipped) gives the node-wise matrix to rounding, and the
    all-core node-wise sparsity equals the edge-sort sparsity."""
    from arcanefem_gb300 import meshgen
    for m, kind in ((meshgen.unit_square_tri(9, seed=3), O.POISSON_TRI3), (meshgen.unit_cube_tet(4, seed=3),
                                                                           O.POISSON_TET4)):
        ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
        rp, cols = O.sparsity(m.nb_node, m.cells)
        ref = O.assemble(kind, m.coords, m.cells, ptr, nc, rp, cols)
        drp, dcols, dvals = O.assemble_dok(kind, m.nb_node, m.coords, m.cells)
        full = np.zeros(cols.size)
        row = np.repeat(np.arange(m.nb_node), np.diff(drp))
        for r, c, v in zip(row, dcols, dvals):
            k = rp[r] + int(np.searchsorted(cols[rp[r]:rp[r + 1]], c))
            assert cols[k] == c
            full[k] = v
        assert np.allclose(full, ref, rtol=1e-12, atol=1e-14 * np.abs(ref).max())
        for t in (1, 4):
            nrp, ncols = O.sparsity_nodewise(m.nb_node, m.cells, ptr, nc, nb_threads=t)
            assert np.array_equal(nrp, rp) and np.array_equal(ncols, cols)
