"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Tolerances:
  * structure (node->cell adjacency, row pointers, columns): bit-exact;
  * matrix values in the default (reference-rounding) and testlab
    formulations: bit-exact (np.array_equal) against the oracle, which
    restates the reference's operation order;
  * matrix values in the minimal-instruction formulation: |a - b| <= 1e-12 *
    max(|b|, 1e-3 * max|row of b|) per entry on these small meshes (its
    element math is regrouped for FP64 throughput, so the last bits differ;
    the guard covers entries that cancel to ~0);
  * Dirichlet transformations on equal inputs: bit-exact;
  * solutions: true FP64 relative residual below the requested tolerance and
    the reference check files within their own tolerance.
"""
import numpy as np
import pytest
import torch

import golden_cases as G
from arcanefem_gb300 import fem, meshgen
from oracle import oracle as O
from parity_helpers import REL, assert_bit_exact, rel_err_rows

pytestmark = pytest.mark.gpu


def build_format(ctx, mesh, nb_dof=1, use_csr=True, col_order=fem.COLS_ASCENDING):
    dm = fem.Mesh.from_host(mesh.dim, mesh.coords, mesh.cells)
    f = fem.BSRFormat(ctx, dm)
    f.initialize(nb_dof, use_csr, col_order)
    f.compute_sparsity()
    return f


MESHES = {
    "tri_4": lambda: meshgen.unit_square_tri(4, seed=1),
    "tri_33": lambda: meshgen.unit_square_tri(33, seed=2),
    "tet_3": lambda: meshgen.unit_cube_tet(3, seed=3),
    "tet_9": lambda: meshgen.unit_cube_tet(9, seed=4),
}


@pytest.mark.parametrize("name", list(MESHES))
def test_node_cell_adjacency_bit_exact(cuda_ctx, name):
    m = MESHES[name]()
    f = build_format(cuda_ctx, m)
    ptr, nc, loc = O.node_cell(m.nb_node, m.cells)
    assert np.array_equal(f.nc_ptr.cpu().numpy(), ptr)
    assert np.array_equal(f.nc_cell.cpu().numpy(), nc)
    assert np.array_equal(f.nc_local.cpu().numpy(), loc)


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("self_last", [False, True])
def test_sparsity_bit_exact(cuda_ctx, name, self_last):
    m = MESHES[name]()
    order = fem.COLS_SELF_LAST if self_last else fem.COLS_ASCENDING
    f = build_format(cuda_ctx, m, col_order=order)
    rp, cols = O.sparsity(m.nb_node, m.cells, self_last=self_last)
    assert np.array_equal(f.row_ptr.cpu().numpy(), rp)
    assert np.array_equal(f.cols.cpu().numpy(), cols)
    assert f.nnzb == meshgen.nnz_formula(m)
    # slot map: for each incidence, slot byte 0 is the row's own column, then the
    # other cell nodes in increasing local index (the order of the element rows)
    slot = f.nc_slot.cpu().numpy().reshape(-1, m.npc)
    ptr, nc, loc = O.node_cell(m.nb_node, m.cells)
    node_of = np.repeat(np.arange(m.nb_node), np.diff(ptr))
    got_cols = cols[rp[node_of][:, None] + slot]
    cell_nodes = m.cells[nc]
    others = np.array([np.delete(row, li) for row, li in zip(cell_nodes, loc)])
    expected = np.concatenate([node_of[:, None], others], axis=1)
    assert np.array_equal(got_cols, expected)


@pytest.mark.parametrize("self_last", [False, True])
def test_sparsity_cols_finds_rows_itself_after_another_meshs_rows(cuda_ctx, self_last):
    """afem_sparsity_cols copies the rows that afem_sparsity_rows kept only when
    it is given the same mesh arrays; after a rows call on another mesh it runs
    the full pass on its own.  Structure and slot map bit-exact both ways, and
    again for the second mesh, whose kept rows the first call left alone."""
    import ctypes as C

    from arcanefem_gb300._capi import call
    order = fem.COLS_SELF_LAST if self_last else fem.COLS_ASCENDING
    ms = [MESHES["tet_9"](), MESHES["tet_3"]()]
    fs = []
    for m in ms:
        f = fem.BSRFormat(cuda_ctx, fem.Mesh.from_host(m.dim, m.coords, m.cells))
        f.initialize(1, col_order=order)
        f.row_ptr = torch.empty(m.nb_node + 1, dtype=torch.int32, device="cuda")
        fs.append(f)
    p = lambda t: C.c_void_p(t.data_ptr())
    nnz = []
    for f in fs:
        k = C.c_int64()
        call("afem_sparsity_rows", cuda_ctx.handle, f.mesh.nb_node, f.mesh.npc, p(f.mesh.cells), p(f.nc_ptr),
             p(f.nc_cell), p(f.row_ptr), C.byref(k))
        nnz.append(int(k.value))
    for f, k, m in zip(fs, nnz, ms):   # the first mesh's rows are no longer kept
        cols = torch.empty(k, dtype=torch.int32, device="cuda")
        slot = torch.empty(m.nb_cell * m.npc * m.npc, dtype=torch.uint8, device="cuda")
        call("afem_sparsity_cols", cuda_ctx.handle, m.nb_node, m.npc, p(f.mesh.cells), p(f.nc_ptr), p(f.nc_cell),
             p(f.nc_local), p(f.row_ptr), order, p(cols), p(slot))
        rp, ref = O.sparsity(m.nb_node, m.cells, self_last=self_last)
        assert np.array_equal(f.row_ptr.cpu().numpy(), rp) and np.array_equal(cols.cpu().numpy(), ref)
        ptr, nc, loc = O.node_cell(m.nb_node, m.cells)
        node_of = np.repeat(np.arange(m.nb_node), np.diff(ptr))
        got = ref[rp[node_of][:, None] + slot.cpu().numpy().reshape(-1, m.npc)]
        others = np.array([np.delete(row, li) for row, li in zip(m.cells[nc], loc)])
        assert np.array_equal(got, np.concatenate([node_of[:, None], others], axis=1))


@pytest.mark.parametrize("self_last", [False, True])
def test_dense_triangle_sparsity_matches_oracle(cuda_ctx, self_last):
    """700 random triangles on 100 nodes: about 21 cells per node, so the
    triangle mesh takes the dense path (8 lanes per node, the nodes in more
    than 32 cells passed on to the warp kernel), with rows of 30 to 50 entries
    (the ranking's general path).  Structure and slot map bit-exact."""
    rng = np.random.default_rng(33)
    n = 100
    cells = np.array([rng.choice(n, 3, replace=False) for _ in range(700)], dtype=np.int32)
    coords = np.concatenate([rng.random((n, 2)), np.zeros((n, 1))], axis=1)
    ptr, nc, loc = O.node_cell(n, cells)
    deg = np.diff(ptr)
    assert deg.mean() > 16 and (deg > 32).any() and (deg <= 32).any()
    f = fem.BSRFormat(cuda_ctx, fem.Mesh.from_host(2, coords, cells))
    f.initialize(1, col_order=fem.COLS_SELF_LAST if self_last else fem.COLS_ASCENDING)
    f.compute_sparsity()
    rp, cols = O.sparsity(n, cells, self_last=self_last)
    assert np.array_equal(f.row_ptr.cpu().numpy(), rp) and np.array_equal(f.cols.cpu().numpy(), cols)
    node_of = np.repeat(np.arange(n), deg)
    got = cols[rp[node_of][:, None] + f.nc_slot.cpu().numpy().reshape(-1, 3)]
    others = np.array([np.delete(row, li) for row, li in zip(cells[nc], loc)])
    assert np.array_equal(got, np.concatenate([node_of[:, None], others], axis=1))


def test_cell_repeating_a_node_keeps_distinct_columns(cuda_ctx):
    """A cell that lists a node twice (a degenerate cell, which the assembly
    reports as such).  Its two incidences of that node number their slot bytes
    by their own local index, which only the node -> cell local indices tell
    apart: the rows pass flags the cell and the columns pass finds the rows
    again with those indices.  Each row holds its node and the distinct nodes
    of its cells; the reference's edge sort (the oracle) would also count the
    repeated node's self-edge, two more entries here."""
    m = MESHES["tet_3"]()
    cells = m.cells.copy()
    cells[5, 2] = cells[5, 1]
    f = fem.BSRFormat(cuda_ctx, fem.Mesh.from_host(3, m.coords, cells))
    f.initialize(1)
    f.compute_sparsity()
    rows = [set([n]) for n in range(m.nb_node)]
    for c in cells:
        for a in c:
            rows[a].update(int(x) for x in c)
    rp = np.concatenate([[0], np.cumsum([len(r) for r in rows])])
    cols = np.concatenate([sorted(r) for r in rows])
    assert np.array_equal(f.row_ptr.cpu().numpy(), rp) and np.array_equal(f.cols.cpu().numpy(), cols)
    assert rp[-1] + 2 == O.sparsity(m.nb_node, cells)[0][-1]
    ptr, nc, loc = O.node_cell(m.nb_node, cells)
    node_of = np.repeat(np.arange(m.nb_node), np.diff(ptr))
    got = cols[rp[node_of][:, None] + f.nc_slot.cpu().numpy().reshape(-1, 4)]
    others = np.array([np.delete(row, li) for row, li in zip(cells[nc], loc)])
    assert np.array_equal(got, np.concatenate([node_of[:, None], others], axis=1))


@pytest.fixture
def formulation_ctx(cuda_ctx):
    """The shared context; the formulation a test sets is put back afterwards."""
    yield cuda_ctx
    cuda_ctx.formulation = fem.FORMULATION_REFERENCE


@pytest.mark.parametrize("name", list(MESHES))
@pytest.mark.parametrize("self_last", [False, True])
def test_poisson_values_match_oracle(formulation_ctx, name, self_last):
    ctx = formulation_ctx
    m = MESHES[name]()
    f = build_format(ctx, m, col_order=fem.COLS_SELF_LAST if self_last else fem.COLS_ASCENDING)
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    rp, cols = O.sparsity(m.nb_node, m.cells, self_last=self_last)
    kind = O.POISSON_TRI3 if m.dim == 2 else O.POISSON_TET4
    kind_t = O.TESTLAB_TRI3 if m.dim == 2 else O.TESTLAB_TET4
    ref = O.assemble(kind, m.coords, m.cells, ptr, nc, rp, cols)
    ref_t = O.assemble(kind_t, m.coords, m.cells, ptr, nc, rp, cols)
    # default: the module formulation in the reference's rounding, bit for bit
    assert ctx.formulation == fem.FORMULATION_REFERENCE
    f.assemble_poisson()
    assert_bit_exact(f.values.cpu().numpy(), ref, "reference formulation")
    # testlab B-matrix formulation (signed measure), bit for bit
    ctx.formulation = fem.FORMULATION_TESTLAB
    f.assemble_poisson()
    assert_bit_exact(f.values.cpu().numpy(), ref_t, "testlab formulation")
    # minimal-instruction formulation: within the guard of both
    ctx.formulation = fem.FORMULATION_MINIMAL
    f.assemble_poisson()
    got = f.values.cpu().numpy()
    assert rel_err_rows(got, ref, rp) < REL
    assert rel_err_rows(got, ref_t, rp) < REL


@pytest.mark.parametrize("formulation", [fem.FORMULATION_REFERENCE, fem.FORMULATION_MINIMAL])
@pytest.mark.parametrize("dim", [2, 3])
def test_poisson_variable_coefficient(formulation_ctx, formulation, dim):
    m = meshgen.unit_square_tri(20, seed=9) if dim == 2 else meshgen.unit_cube_tet(6, seed=9)
    k = np.exp(np.random.default_rng(0).standard_normal(m.nb_cell))
    formulation_ctx.formulation = formulation
    f = build_format(formulation_ctx, m)
    f.assemble_poisson(torch.as_tensor(k, device="cuda"))
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    rp, cols = O.sparsity(m.nb_node, m.cells)
    ref = O.assemble(O.POISSON_TRI3 if dim == 2 else O.POISSON_TET4, m.coords, m.cells, ptr, nc, rp, cols,
                     cell_coeff=k)
    if formulation == fem.FORMULATION_REFERENCE:
        assert_bit_exact(f.values.cpu().numpy(), ref, "coefficient")
    else:
        assert rel_err_rows(f.values.cpu().numpy(), ref, rp) < REL


@pytest.mark.parametrize("formulation", [fem.FORMULATION_REFERENCE, fem.FORMULATION_MINIMAL])
@pytest.mark.parametrize("use_csr", [True, False])
def test_elasticity_values_match_oracle(formulation_ctx, use_csr, formulation):
    m = meshgen.unit_cube_tet(5, seed=6)
    lam, mu = fem.lame(21e5, 0.28)
    formulation_ctx.formulation = formulation
    f = build_format(formulation_ctx, m, nb_dof=3, use_csr=use_csr)
    f.assemble_elasticity(lam, mu)
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    rp, cols = O.sparsity(m.nb_node, m.cells)
    ref = O.assemble(O.ELASTICITY_TET4, m.coords, m.cells, ptr, nc, rp, cols, per_block_layout=not use_csr,
                     lam=lam, mu=mu)
    got = f.values.cpu().numpy()
    if formulation == fem.FORMULATION_REFERENCE:
        assert_bit_exact(got, ref, "elasticity")
    elif use_csr:
        srp, _ = G.scalar_csr_from_block(rp, cols, 3)
        assert rel_err_rows(got, ref, srp) < REL
    else:
        assert rel_err_rows(got, ref, rp, b=3) < REL


def test_bsr_to_csr_structure(cuda_ctx):
    m = meshgen.unit_cube_tet(3, seed=1)
    f = build_format(cuda_ctx, m, nb_dof=3)
    srp, scols, _ = f.to_csr()
    rp, cols = O.sparsity(m.nb_node, m.cells)
    erp, ecols = G.scalar_csr_from_block(rp, cols, 3)
    assert np.array_equal(srp.cpu().numpy(), erp) and np.array_equal(scols.cpu().numpy(), ecols)


def test_assembly_is_deterministic(cuda_ctx):
    m = meshgen.unit_cube_tet(8, seed=11)
    f = build_format(cuda_ctx, m)
    f.assemble_poisson()
    a = f.values.clone()
    f.reset_matrix_values()
    f.assemble_poisson()
    assert torch.equal(a, f.values)


@pytest.mark.parametrize("dim", [2, 3])
def test_rhs_constant_source(cuda_ctx, dim):
    m = meshgen.unit_square_tri(12, seed=1) if dim == 2 else meshgen.unit_cube_tet(4, seed=1)
    f = build_format(cuda_ctx, m)
    rhs = torch.zeros(m.nb_node, dtype=torch.float64, device="cuda")
    f.rhs_constant_source(-5.5, rhs)
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    ref = O.rhs_constant_source(dim, m.coords, m.cells, ptr, nc, -5.5)
    assert_bit_exact(rhs.cpu().numpy(), ref, "constant source")


def test_rhs_body_force(cuda_ctx):
    m = meshgen.unit_cube_tet(4, seed=2)
    f = build_format(cuda_ctx, m, nb_dof=3)
    rhs = torch.zeros(3 * m.nb_node, dtype=torch.float64, device="cuda")
    f.rhs_body_force([0.0, 0.5, -1.0], rhs)
    ref = O.rhs_body_force_tet4(m.coords, m.cells, [0.0, 0.5, -1.0])
    assert_bit_exact(rhs.cpu().numpy(), ref, "body force")


def test_dirichlet_transformations_bit_exact(cuda_ctx):
    m = meshgen.unit_square_tri(6, seed=3)
    f = build_format(cuda_ctx, m)
    f.assemble_poisson()
    rp, cols, vals = (t.cpu().numpy() for t in f.to_csr())
    n = m.nb_node
    rng = np.random.default_rng(5)
    rhs0 = rng.standard_normal(n)
    ls = fem.DoFLinearSystem(cuda_ctx, n)
    f.to_linear_system(ls)
    ls.rhs_variable().copy_(torch.as_tensor(rhs0))
    dev = lambda a: torch.as_tensor(np.asarray(a, np.int32), device="cuda")  # noqa: E731
    ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, dev([0, 5, 9]), 1, 0, 0.25)
    ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW, dev([14, 15]), 1, 0, -1.5)
    ls.apply_dirichlet_penalty(dev([30, 31]), 1, 0, 2.0, 1e30)
    ls.apply_matrix_transformation()
    ls.apply_rhs_transformation()
    # oracle on the same inputs
    fi, fv = np.zeros(n, np.uint8), np.zeros(n)
    ei, ev = np.zeros(n, np.uint8), np.zeros(n)
    rr = rhs0.copy()
    O.dirichlet_elimination(np.array([0, 5, 9]), 1, 0, 0.25, 2, ei, ev)
    O.dirichlet_elimination(np.array([14, 15]), 1, 0, -1.5, 1, ei, ev)
    O.dirichlet_penalty(np.array([30, 31]), 1, 0, 2.0, 1e30, fi, fv, rr)
    vv = vals.copy()
    O.apply_transformations(rp, cols, vv, rr, fi, fv, ei, ev)
    assert np.array_equal(f.values.cpu().numpy(), vv)
    assert np.array_equal(ls.rhs_variable().cpu().numpy(), rr)
    assert np.array_equal(ls.get_forced_info().cpu().numpy(), fi)
    assert np.array_equal(ls.get_elimination_info().cpu().numpy(), ei)


def test_linear_system_entry_api(cuda_ctx):
    m = meshgen.unit_square_tri(3, seed=0)
    f = build_format(cuda_ctx, m)
    f.assemble_poisson()
    ls = fem.DoFLinearSystem(cuda_ctx, m.nb_node)
    f.to_linear_system(ls)
    before = f.values.clone()
    ls.matrix_add_value(0, 0, 1.5)
    ls.matrix_set_value(1, 1, 7.0)
    rp = f.row_ptr.cpu().numpy()
    cols = f.cols.cpu().numpy()
    k00 = rp[0] + list(cols[rp[0]:rp[1]]).index(0)
    k11 = rp[1] + list(cols[rp[1]:rp[2]]).index(1)
    assert f.values[k00].item() == before[k00].item() + 1.5 and f.values[k11].item() == 7.0
    with pytest.raises(fem.AfemError) as e:
        ls.matrix_add_value(0, m.nb_node - 1, 1.0)     # not in the sparsity
    assert e.value.status == 9
    with pytest.raises(fem.AfemError) as e:
        ls.eliminate_row(0, 1.0)
    assert e.value.status == 8


@pytest.mark.parametrize("precision", [fem.PRECISION_FP64, fem.PRECISION_MIXED])
def test_cg_solution_matches_oracle(cuda_ctx, precision):
    m = meshgen.unit_cube_tet(10, seed=4)
    f = build_format(cuda_ctx, m)
    f.assemble_poisson()
    ls = fem.DoFLinearSystem(cuda_ctx, m.nb_node)
    f.to_linear_system(ls)
    f.rhs_constant_source(1.0, ls.rhs_variable())
    nodes = torch.as_tensor(m.groups["x_faces"], device="cuda")
    ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, nodes, 1, 0, 0.0)
    info = ls.apply_linear_system_transformation_and_solve(
        fem.solver_options(rtol=1e-10, max_iter=5000, precision=precision))
    assert info.status == 0 and info.relres < 1e-10
    # oracle solution of the same transformed system
    rp, cols, vals = (t.cpu().numpy() for t in f.to_csr())
    b = ls.rhs_variable().cpu().numpy()
    x_ref, _, _ = O.pcg_jacobi(rp, cols, vals, b, rtol=1e-13, max_iter=20000)
    x = ls.solution_variable().cpu().numpy()
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-8
    if precision == fem.PRECISION_MIXED:
        assert info.refinements >= 1


def test_mixed_precision_iterations_stay_close_to_fp64(cuda_ctx):
    """Mixed precision keeps its FP32 CG direction across the reliable updates
    (true FP64 residual every decade), so on a 128^2 Poisson problem to 1e-8
    its FP32 iterations stay close to the FP64 CG's instead of growing with
    every restart."""
    m = meshgen.unit_square_tri(128, seed=5)
    f = build_format(cuda_ctx, m)
    f.assemble_poisson()
    rp, cols, vals = f.to_csr()
    ls = fem.DoFLinearSystem(cuda_ctx, m.nb_node)
    f.to_linear_system(ls)
    f.rhs_constant_source(-1.0, ls.rhs_variable())
    nodes = torch.as_tensor(m.groups["boundary"], device="cuda")
    ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, nodes, 1, 0, 0.0)
    ls.apply_matrix_transformation()
    ls.apply_rhs_transformation()
    b = ls.rhs_variable().clone()
    its = {}
    for prec in (fem.PRECISION_FP64, fem.PRECISION_MIXED):
        x = torch.zeros_like(b)
        info = fem.cg_solve_csr(cuda_ctx, rp, cols, vals, b, x,
                                options=fem.solver_options(rtol=1e-8, max_iter=20000, precision=prec,
                                                           inner_rtol=0.1))
        assert info.status == 0 and info.relres < 1e-8
        its[prec] = (info.iterations, info.refinements)
    print("iterations (FP32 CG, reliable updates) vs FP64 CG", its)
    assert its[fem.PRECISION_MIXED][1] >= 6, its         # one update per decade
    assert its[fem.PRECISION_MIXED][0] <= 1.3 * its[fem.PRECISION_FP64][0], its


def test_cg_penalty_with_skipped_forced_rows(cuda_ctx):
    m = meshgen.unit_square_tri(24, seed=2)
    f = build_format(cuda_ctx, m)
    f.assemble_poisson()
    ls = fem.DoFLinearSystem(cuda_ctx, m.nb_node)
    f.to_linear_system(ls)
    f.rhs_constant_source(-1.0, ls.rhs_variable())
    ls.apply_dirichlet_penalty(torch.as_tensor(m.groups["boundary"], device="cuda"), 1, 0, 0.5, 1e30)
    info = ls.apply_linear_system_transformation_and_solve(
        fem.solver_options(rtol=1e-12, max_iter=5000, skip_forced_rows=True))
    assert info.status == 0 and info.relres < 1e-12
    x = ls.solution_variable().cpu().numpy()
    assert np.allclose(x[m.groups["boundary"]], 0.5, rtol=0, atol=1e-12)


def test_spmv_matches_oracle(cuda_ctx):
    m = meshgen.unit_cube_tet(6, seed=8)
    f = build_format(cuda_ctx, m, nb_dof=3)
    f.assemble_elasticity(*fem.lame(1.0, 0.3))
    rp, cols, vals = f.to_csr()
    x = torch.randn(3 * m.nb_node, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    fem.spmv_csr(cuda_ctx, rp, cols, vals, x, y)
    ref = O.spmv(rp.cpu().numpy(), cols.cpu().numpy(), vals.cpu().numpy(), x.cpu().numpy())
    np.testing.assert_allclose(y.cpu().numpy(), ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("name", list(G.CASES))
def test_golden_case_on_gpu(cuda_ctx, name):
    """The reference test cases end to end on the GPU path, compared with the
    reference's own check files."""
    spec = G.CASES[name]
    d = G.load(name)
    dim = 2 if d["cells"].shape[1] == 3 else 3
    mesh = meshgen.Mesh(dim, d["coords"], d["cells"])
    if spec["kind"] == "elasticity":
        f = build_format(cuda_ctx, mesh, nb_dof=3)
        f.assemble_elasticity(*fem.lame(spec["E"], spec["nu"]))
        ls = fem.DoFLinearSystem(cuda_ctx, 3 * mesh.nb_node)
        f.to_linear_system(ls)
        f.rhs_body_force(spec["body_force"], ls.rhs_variable())
        for g, v3 in spec["dirichlet3"]:
            for comp, v in enumerate(v3):
                if v is not None:
                    ls.apply_dirichlet_penalty(torch.as_tensor(d["group__" + g], device="cuda"), 3, comp, v,
                                               spec["penalty"])
    else:
        f = build_format(cuda_ctx, mesh)
        f.assemble_poisson()
        ls = fem.DoFLinearSystem(cuda_ctx, mesh.nb_node)
        f.to_linear_system(ls)
        f.rhs_constant_source(spec["f"], ls.rhs_variable())
        for g, v in spec["dirichlet"]:
            ls.apply_dirichlet_penalty(torch.as_tensor(d["group__" + g], device="cuda"), 1, 0, v, spec["penalty"])
    info = ls.apply_linear_system_transformation_and_solve(
        fem.solver_options(rtol=1e-12, max_iter=20000, skip_forced_rows=True))
    err = G.compare(name, ls.solution_variable().cpu().numpy(), d)
    assert err < spec["eps"], f"{name}: {err:.3e} (iters {info.iterations}, relres {info.relres:.2e})"


def test_bad_mesh_is_reported(cuda_ctx):
    m = meshgen.unit_square_tri(2)
    cells = m.cells.copy()
    cells[0, 0] = m.nb_node + 5            # out of range: caught by the kernel's own bounds check
    dm = fem.Mesh.from_host(2, m.coords, cells)
    f = fem.BSRFormat(cuda_ctx, dm)
    with pytest.raises(fem.AfemError) as e:
        f.initialize(1)
    assert e.value.status == 7


def test_single_cell_meshes(cuda_ctx):
    for dim, coords, cells in ((2, [[0, 0, 0], [1, 0, 0], [0, 1, 0]], [[0, 1, 2]]),
                               (3, [[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], [[0, 1, 2, 3]])):
        m = meshgen.Mesh(dim, np.array(coords, float), np.array(cells, np.int32))
        f = build_format(cuda_ctx, m)
        f.assemble_poisson()
        n = dim + 1
        assert f.nnzb == n * n
        K = f.values.cpu().numpy().reshape(n, n)
        ref = np.array([O.elem_vec(O.POISSON_TRI3 if dim == 2 else O.POISSON_TET4, m.coords, cells[0], i)
                        for i in range(n)])
        np.testing.assert_allclose(K, ref, rtol=1e-14, atol=1e-15)


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("mode", [fem.FACE_SCALAR, fem.FACE_NORMAL, fem.FACE_VECTOR])
def test_boundary_face_terms_bit_exact(cuda_ctx, dim, mode):
    """Neumann (scalar / normal flux) and traction terms: the GPU's node-wise
    gather in increasing face order equals the oracle's sequential face loop
    bit for bit, added into an existing right-hand side."""
    m = meshgen.unit_square_tri(40, seed=7) if dim == 2 else meshgen.unit_cube_tet(12, seed=7)
    f, out = meshgen.boundary_faces(m, seed=11)
    nb_dof = dim if mode == fem.FACE_VECTOR else 1
    g = [0.75, -1.25, 2.0][:dim] if mode != fem.FACE_SCALAR else [-5.5]
    rhs0 = np.random.default_rng(1).standard_normal(m.nb_node * nb_dof)
    ref = O.rhs_boundary_faces(dim, m.coords, f, out, mode, g, nb_dof, rhs0.copy())
    co = torch.as_tensor(m.coords, device="cuda")
    fd = torch.as_tensor(f, device="cuda")
    od = torch.as_tensor(out, device="cuda")
    rhs = torch.as_tensor(rhs0, device="cuda")
    fem.rhs_boundary_faces(cuda_ctx, dim, co, fd, od, mode, g, nb_dof, rhs)
    assert np.array_equal(rhs.cpu().numpy(), ref)


Q1_MESHES = {
    "quad_7": lambda: meshgen.unit_square_quad(7, seed=5),
    "quad_40": lambda: meshgen.unit_square_quad(40, seed=6),
    "hex_3": lambda: meshgen.unit_cube_hex(3, seed=7),
    "hex_10": lambda: meshgen.unit_cube_hex(10, seed=8),
}


@pytest.mark.parametrize("name", list(Q1_MESHES))
def test_q1_structure_and_values_match_oracle(cuda_ctx, name):
    """Quad4 / Hexa8 (bilinear / trilinear Lagrange, 2x2(x2) Gauss points):
    node -> cell incidence and sparsity bit-exact; values bit-exact in the
    reference formulation, within 1e-12 per entry in the minimal one, against
    the oracle's node-wise assembly of the reference element vectors."""
    m = Q1_MESHES[name]()
    f = build_format(cuda_ctx, m)
    ptr, nc, loc = O.node_cell(m.nb_node, m.cells)
    assert np.array_equal(f.nc_ptr.cpu().numpy(), ptr) and np.array_equal(f.nc_cell.cpu().numpy(), nc)
    assert np.array_equal(f.nc_local.cpu().numpy(), loc)
    rp, cols = O.sparsity(m.nb_node, m.cells)
    assert np.array_equal(f.row_ptr.cpu().numpy(), rp) and np.array_equal(f.cols.cpu().numpy(), cols)
    k = torch.as_tensor(np.exp(np.random.default_rng(2).standard_normal(m.nb_cell)), device="cuda")
    f.assemble_poisson(k)
    kind = O.POISSON_QUAD4 if m.dim == 2 else O.POISSON_HEXA8
    ref = O.assemble(kind, m.coords, m.cells, ptr, nc, rp, cols, cell_coeff=k.cpu().numpy())
    assert_bit_exact(f.values.cpu().numpy(), ref, "Q1 reference formulation")
    cuda_ctx.formulation = fem.FORMULATION_MINIMAL
    try:
        f.assemble_poisson(k)
    finally:
        cuda_ctx.formulation = fem.FORMULATION_REFERENCE
    assert rel_err_rows(f.values.cpu().numpy(), ref, rp) < REL


@pytest.mark.parametrize("dim", [2, 3])
def test_q1_constant_source(cuda_ctx, dim):
    m = meshgen.unit_square_quad(17, seed=3) if dim == 2 else meshgen.unit_cube_hex(6, seed=3)
    f = build_format(cuda_ctx, m)
    rhs = torch.zeros(m.nb_node, dtype=torch.float64, device="cuda")
    f.rhs_constant_source(-5.5, rhs)
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    ref = O.rhs_constant_source_q1(dim, m.coords, m.cells, ptr, nc, -5.5)
    assert_bit_exact(rhs.cpu().numpy(), ref, "Q1 constant source")


def test_q1_poisson_solve(cuda_ctx):
    """Hexa8 assembly + Q1 source + row-column elimination + CG to 1e-10,
    against the oracle's CG on the oracle's system."""
    m = meshgen.unit_cube_hex(8, seed=4)
    f = build_format(cuda_ctx, m)
    f.assemble_poisson()
    ls = fem.DoFLinearSystem(cuda_ctx, m.nb_node)
    f.to_linear_system(ls)
    f.rhs_constant_source(1.0, ls.rhs_variable())
    nodes = torch.as_tensor(m.groups["x_faces"], device="cuda")
    ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, nodes, 1, 0, 0.0)
    info = ls.apply_linear_system_transformation_and_solve(fem.solver_options(rtol=1e-10, max_iter=5000))
    assert info.status == 0 and info.relres < 1e-10
    rp, cols, vals = (t.cpu().numpy() for t in f.to_csr())
    x_ref, _, _ = O.pcg_jacobi(rp, cols, vals, ls.rhs_variable().cpu().numpy(), rtol=1e-13, max_iter=20000)
    x = ls.solution_variable().cpu().numpy()
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-8


def test_msh_to_vtu_end_to_end(cuda_ctx, tmp_path):
    """gmsh MSH 4.1 in (written from a synthetic mesh), assembly + source +
    row-column Dirichlet + CG on the GPU, VTU out; the solution equals the
    one obtained from the in-memory mesh."""
    import xml.etree.ElementTree as ET

    from arcanefem_gb300 import meshio
    from arcanefem_gb300.examples import poisson_msh
    m = meshgen.unit_square_tri(20, seed=9)
    path = str(tmp_path / "sq.msh")
    meshio.write_msh(path, m)
    d, u, info = poisson_msh.solve(path, -5.5, {"boundary": 0.5}, ctx=cuda_ctx)
    assert info.status == 0 and info.relres < 1e-10
    assert np.allclose(u[m.groups["boundary"]], 0.5)
    out = str(tmp_path / "u.vtu")
    meshio.write_vtu(out, d.mesh, point_data={"U": u})
    assert int(ET.parse(out).getroot().find("UnstructuredGrid/Piece").get("NumberOfPoints")) == m.nb_node
    # the same problem from the in-memory mesh (penalty, the module's default)
    f = build_format(cuda_ctx, m)
    f.assemble_poisson()
    ls = fem.DoFLinearSystem(cuda_ctx, m.nb_node)
    f.to_linear_system(ls)
    f.rhs_constant_source(-5.5, ls.rhs_variable())
    ls.apply_dirichlet_penalty(torch.as_tensor(m.groups["boundary"], device="cuda"), 1, 0, 0.5, 1e30)
    ls.apply_linear_system_transformation_and_solve(
        fem.solver_options(rtol=1e-10, max_iter=100000, skip_forced_rows=True))
    assert np.allclose(ls.solution_variable().cpu().numpy(), u, rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("case", ["tri", "tet", "quad", "hex", "elast_block", "elast_row"])
@pytest.mark.parametrize("chunks", [0, 1, 3, 16])
def test_gather_to_host_matches_device_gather(cuda_ctx, case, chunks):
    """The chunked gather with overlapped copies back to a host buffer gives
    exactly the values of the one-shot device gather."""
    mesh = {"tri": lambda: meshgen.unit_square_tri(20, seed=1), "tet": lambda: meshgen.unit_cube_tet(7, seed=2),
            "quad": lambda: meshgen.unit_square_quad(13, seed=3), "hex": lambda: meshgen.unit_cube_hex(5, seed=4),
            "elast_block": lambda: meshgen.unit_cube_tet(5, seed=5),
            "elast_row": lambda: meshgen.unit_cube_tet(5, seed=6)}[case]()
    nb_dof = 3 if case.startswith("elast") else 1
    f = build_format(cuda_ctx, mesh, nb_dof=nb_dof, use_csr=(case != "elast_block"))
    ke = torch.empty(f.element_buffer_size(), dtype=torch.float64, device="cuda")
    f.element_matrices(ke, lam=1.3, mu=0.7)
    f.gather(ke)
    ref = f.values.cpu().clone()
    f.values.fill_(float("nan"))
    host = torch.full((f.values.numel(),), float("nan"), dtype=torch.float64).pin_memory()
    f.gather_to_host(ke, host, chunks=chunks)
    assert torch.equal(host, ref)
    assert torch.equal(f.values.cpu(), ref)


def test_mixed_bsr_spmv_solves_elasticity(cuda_ctx):
    """Elasticity (3 DoF per node): the mixed solver with the FP32 3x3-block
    SpMV (block_size 3, set by the BSRFormat's linear system) reaches the FP64
    residual target, and its solution matches the scalar-CSR mixed solve and
    the FP64 solve."""
    m = meshgen.unit_cube_tet(8, seed=7)
    sols = {}
    for tag, prec, block in (("fp64", fem.PRECISION_FP64, 0), ("mixed_csr", fem.PRECISION_MIXED, 1),
                             ("mixed_bsr", fem.PRECISION_MIXED, 0)):
        f = build_format(cuda_ctx, m, nb_dof=3)
        lam, mu = fem.lame(21e5, 0.28)
        f.assemble_elasticity(lam, mu)
        ls = fem.DoFLinearSystem(cuda_ctx, 3 * m.nb_node)
        f.to_linear_system(ls)
        f.rhs_body_force((0.0, 0.0, -1.0), ls.rhs_variable())
        nodes = torch.as_tensor(m.groups["zmin"], device="cuda")
        for comp in range(3):
            ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, nodes, 3, comp, 0.0)
        info = ls.apply_linear_system_transformation_and_solve(
            fem.solver_options(rtol=1e-8, max_iter=20000, precision=prec, block_size=block))
        assert info.status == 0 and info.relres < 1e-8, (tag, info.relres)
        sols[tag] = ls.solution_variable().clone()
    ref = sols["fp64"]
    for tag in ("mixed_csr", "mixed_bsr"):
        assert torch.linalg.norm(sols[tag] - ref) <= 1e-6 * torch.linalg.norm(ref), tag


def test_mixed_bsr_rejects_a_scalar_pattern(cuda_ctx):
    m = meshgen.unit_square_tri(9, seed=1)
    f = build_format(cuda_ctx, m)
    f.assemble_poisson()
    rp, cols, vals = f.to_csr()
    n = m.nb_node - m.nb_node % 3
    rp3 = rp[:n + 1].contiguous()
    b = torch.ones(n, dtype=torch.float64, device="cuda")
    x = torch.zeros_like(b)
    with pytest.raises(fem.AfemError) as e:
        fem.cg_solve_csr(cuda_ctx, rp3, cols, vals, b, x,
                         options=fem.solver_options(precision=fem.PRECISION_MIXED, block_size=3))
    assert e.value.status == 1


@pytest.mark.parametrize("case", ["tri", "tet", "quad", "hex", "elast_block", "elast_row"])
@pytest.mark.parametrize("chunks", [0, 1, 4, 16])
@pytest.mark.parametrize("host_coords", [False, True])
def test_assemble_to_host_matches_two_stage_assembly(cuda_ctx, case, chunks, host_coords):
    """The pipelined assembly (cell ranges, the node prefixes they complete
    gathered and copied back behind them) gives exactly the values of the
    element kernel followed by the one-shot gather; with host coordinates
    (afem_assemble_host_io) the device coordinates start as NaN and every
    range must wait for the upload of the nodes its cells use."""
    mesh = {"tri": lambda: meshgen.unit_square_tri(21, seed=1), "tet": lambda: meshgen.unit_cube_tet(7, seed=2),
            "quad": lambda: meshgen.unit_square_quad(13, seed=3), "hex": lambda: meshgen.unit_cube_hex(5, seed=4),
            "elast_block": lambda: meshgen.unit_cube_tet(5, seed=5),
            "elast_row": lambda: meshgen.unit_cube_tet(6, seed=6)}[case]()
    nb_dof = 3 if case.startswith("elast") else 1
    f = build_format(cuda_ctx, mesh, nb_dof=nb_dof, use_csr=(case != "elast_block"))
    coeff = None if nb_dof == 3 else torch.as_tensor(np.exp(np.random.default_rng(3).standard_normal(mesh.nb_cell)),
                                                      device="cuda")
    ke = torch.empty(f.element_buffer_size(), dtype=torch.float64, device="cuda")
    f.element_matrices(ke, cell_coeff=coeff, lam=1.3, mu=0.7)
    f.gather(ke)
    ref = f.values.cpu().clone()
    f.values.fill_(float("nan"))
    ke.fill_(float("nan"))
    host = torch.full((f.values.numel(),), float("nan"), dtype=torch.float64).pin_memory()
    coords_h = None
    if host_coords:
        coords_h = f.mesh.coords.cpu().pin_memory()
        f.mesh.coords.fill_(float("nan"))
    f.assemble_to_host(ke, host, chunks=chunks, cell_coeff=coeff, lam=1.3, mu=0.7, coords_h=coords_h)
    assert torch.equal(host, ref)
    assert torch.equal(f.values.cpu(), ref)
    if host_coords:
        assert torch.equal(f.mesh.coords.cpu(), coords_h)


def fan_mesh(k, isolated=0):
    """k triangles around node 0 (a row of k + 1 entries), plus `isolated`
    nodes that belong to no cell."""
    t = np.linspace(0.0, 2 * np.pi, k, endpoint=False)
    ring = np.stack([np.cos(t), np.sin(t), np.zeros(k)], 1)
    coords = np.concatenate([np.zeros((1, 3)), ring, np.full((isolated, 3), 2.0)], 0)
    cells = np.array([[0, 1 + i, 1 + (i + 1) % k] for i in range(k)], np.int32)
    return coords, cells


@pytest.mark.parametrize("k,isolated", [(12, 0), (40, 0), (100, 2), (200, 1), (254, 0)])
def test_fan_rows_and_isolated_nodes_match_oracle(cuda_ctx, k, isolated):
    """Rows longer than the gather's shared-memory accumulators (the direct
    path: 41 to 255 entries; the hub's incidences span several chunks of 32 in
    the sparsity kernels, and 255 entries is the longest row the uint8 slot map
    addresses) and nodes in no cell (a diagonal-only row, as the reference's
    deg + 1 rows): structure and values bit-exact."""
    coords, cells = fan_mesh(k, isolated)
    n = coords.shape[0]
    f = fem.BSRFormat(cuda_ctx, fem.Mesh.from_host(2, coords, cells))
    f.initialize(1)
    f.compute_sparsity()
    rp, cols = O.sparsity(n, cells)
    assert np.array_equal(f.row_ptr.cpu().numpy(), rp) and np.array_equal(f.cols.cpu().numpy(), cols)
    f.assemble_poisson()
    ptr, nc, _ = O.node_cell(n, cells)
    ref = O.assemble(O.POISSON_TRI3, coords, cells, ptr, nc, rp, cols)
    assert_bit_exact(f.values.cpu().numpy(), ref, "fan rows")


@pytest.mark.parametrize("formulation", [fem.FORMULATION_REFERENCE, fem.FORMULATION_TESTLAB,
                                         fem.FORMULATION_MINIMAL])
@pytest.mark.parametrize("kind", ["tet", "tri", "hex", "elasticity"])
def test_degenerate_cell_is_reported(formulation_ctx, formulation, kind):
    """A cell of zero measure (a flattened tetrahedron / triangle / hexahedron)
    makes its element matrix non-finite; the element kernel flags it and the
    next synchronous call returns AFEM_ERR_MESH, after which the context is
    usable again.  The flag is raised on the host side of the API, not by a
    device fault."""
    ctx = formulation_ctx
    ctx.formulation = formulation
    if kind in ("tet", "elasticity"):
        m = meshgen.unit_cube_tet(3, seed=1)
    elif kind == "tri":
        m = meshgen.unit_square_tri(4, seed=1)
    else:
        m = meshgen.unit_cube_hex(3, seed=1)
    bad = m.coords.copy()
    # move every node of cell 0 onto the plane z = 0 (3D) or the line y = y_0 (2D):
    # its measure is then exactly zero in every formulation
    cn = m.cells[0]
    if m.dim == 3:
        bad[cn, 2] = 0.0
    else:
        bad[cn, 1] = bad[cn[0], 1]
    f = build_format(ctx, meshgen.Mesh(m.dim, bad, m.cells), nb_dof=3 if kind == "elasticity" else 1)
    if kind == "elasticity":
        f.assemble_elasticity(*fem.lame(21e5, 0.28))
    else:
        f.assemble_poisson()
    with pytest.raises(fem.AfemError) as e:
        ctx.synchronize()
    assert e.value.status == 7 and "degenerate cell" in str(e.value)
    ctx.synchronize()   # the flag was cleared
    g = build_format(ctx, m, nb_dof=3 if kind == "elasticity" else 1)
    if kind == "elasticity":
        g.assemble_elasticity(*fem.lame(21e5, 0.28))
    else:
        g.assemble_poisson()
    ctx.synchronize()
    assert torch.isfinite(g.values).all()


def star_mesh(k):
    """k triangles that share only node 0 (a non-manifold star): node 0 is in
    k cells and has 2k distinct neighbours."""
    t = np.linspace(0.0, 2 * np.pi, 2 * k, endpoint=False)
    ring = np.stack([np.cos(t), np.sin(t), np.zeros(2 * k)], 1)
    coords = np.concatenate([np.zeros((1, 3)), ring], 0)
    cells = np.array([[0, 1 + 2 * i, 2 + 2 * i] for i in range(k)], np.int32)
    return coords, cells


@pytest.mark.parametrize("k,self_last", [(8, False), (10, False), (10, True), (16, False), (16, True)])
def test_rows_with_many_neighbours_per_cell_match_oracle(cuda_ctx, k, self_last):
    """A node in at most 16 cells goes to the thread-per-node sparsity kernel,
    which ranks up to 16 neighbours by a sorting network (k = 8) and 17 to 24
    by counting (k = 10: 20 neighbours); with 2k > 24 distinct neighbours
    (k = 16) its row overflows that kernel's table and is deferred to the warp
    kernel through the node list.  Structure, slot map and values bit-exact in
    both column orders."""
    coords, cells = star_mesh(k)
    n = coords.shape[0]
    f = fem.BSRFormat(cuda_ctx, fem.Mesh.from_host(2, coords, cells))
    f.initialize(1, col_order=fem.COLS_SELF_LAST if self_last else fem.COLS_ASCENDING)
    f.compute_sparsity()
    rp, cols = O.sparsity(n, cells, self_last=self_last)
    assert np.array_equal(f.row_ptr.cpu().numpy(), rp) and np.array_equal(f.cols.cpu().numpy(), cols)
    f.assemble_poisson()
    ptr, nc, _ = O.node_cell(n, cells)
    ref = O.assemble(O.POISSON_TRI3, coords, cells, ptr, nc, rp, cols)
    assert_bit_exact(f.values.cpu().numpy(), ref, "star rows")


def delaunay_mesh(dim, npts, seed):
    """Delaunay triangles / tetrahedra of random points in the unit square /
    cube, nodes renumbered at random: uneven degrees (tetrahedra: 8 to over
    60 cells per node, rows of 7 to over 30 entries)."""
    spatial = pytest.importorskip("scipy.spatial")
    rng = np.random.default_rng(seed)
    pts = rng.random((npts, dim))
    cells = spatial.Delaunay(pts).simplices.astype(np.int32)
    perm = rng.permutation(npts).astype(np.int32)
    coords = np.zeros((npts, 3))
    coords[perm, :dim] = pts
    return coords, perm[cells]


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("self_last", [False, True])
@pytest.mark.parametrize("aligned", [True, False])
def test_unstructured_sparsity_matches_oracle(cuda_ctx, dim, self_last, aligned):
    """Unstructured meshes with randomly numbered nodes through both sparsity
    kernels (triangles: a thread per node; tetrahedra, about 26 cells per
    node: a warp per node).  With aligned=False the cell array starts 4 bytes
    past a 16-byte boundary, so the cell nodes are read one by one instead of
    in 16-byte loads.  Structure and slot map bit-exact; values bit-exact with
    the aligned array (the assembly kernels require 16-byte aligned
    cell_nodes)."""
    coords, cells = delaunay_mesh(dim, 4000, seed=21)
    n, npc = coords.shape[0], dim + 1
    rp, cols = O.sparsity(n, cells, self_last=self_last)
    ptr, nc, loc = O.node_cell(n, cells)
    deg = np.diff(ptr)
    buf = torch.zeros(cells.size + 4, dtype=torch.int32, device="cuda")
    off = 0 if aligned else 1
    buf[off:off + cells.size] = torch.as_tensor(cells.reshape(-1), device="cuda")
    ce = buf[off:off + cells.size].view(-1, npc)
    assert (ce.data_ptr() % 16 == 0) == aligned
    mesh = fem.Mesh(dim, torch.as_tensor(coords, device="cuda"), ce)
    f = fem.BSRFormat(cuda_ctx, mesh)
    f.initialize(1, col_order=fem.COLS_SELF_LAST if self_last else fem.COLS_ASCENDING)
    f.compute_sparsity()
    assert np.array_equal(f.row_ptr.cpu().numpy(), rp) and np.array_equal(f.cols.cpu().numpy(), cols)
    slot = f.nc_slot.cpu().numpy().reshape(-1, npc)
    node_of = np.repeat(np.arange(n), deg)
    others = np.array([np.delete(row, li) for row, li in zip(cells[nc], loc)])
    assert np.array_equal(cols[rp[node_of][:, None] + slot], np.concatenate([node_of[:, None], others], axis=1))
    if aligned:
        f.assemble_poisson()
        ref = O.assemble(O.POISSON_TET4 if dim == 3 else O.POISSON_TRI3, coords, cells, ptr, nc, rp, cols)
        assert_bit_exact(f.values.cpu().numpy(), ref, "unstructured mesh")


@pytest.mark.parametrize("k", [255, 300])
def test_row_above_the_slot_map_capacity_is_reported(cuda_ctx, k):
    """A node in k triangles has a row of k + 1 entries; above 255 (the uint8
    slot map) it is reported as a mesh error, not truncated, and the context
    stays usable."""
    coords, cells = fan_mesh(k)
    f = fem.BSRFormat(cuda_ctx, fem.Mesh.from_host(2, coords, cells))
    f.initialize(1)
    with pytest.raises(fem.AfemError) as e:
        f.compute_sparsity()
    assert e.value.status == 7 and "more than 255 entries" in str(e.value)
    coords, cells = fan_mesh(12)
    g = fem.BSRFormat(cuda_ctx, fem.Mesh.from_host(2, coords, cells))
    g.initialize(1)
    g.compute_sparsity()
    assert g.nnzb == 13 + 12 * 4   # the hub row, then 12 rows of 4


def hub_laplacian(n, hubs, seed):
    """SPD CSR with very uneven rows: a random sparse graph Laplacian (weights
    in [0.5, 1.5]) plus hub nodes joined to a third of the graph, shifted by
    0.1 I; rows from 2 to ~n/3 + 2 entries, n not a multiple of 32."""
    rng = np.random.default_rng(seed)
    edges = {(min(i, j), max(i, j)) for i, j in rng.integers(0, n, (3 * n, 2)) if i != j}
    for h in hubs:
        edges |= {(min(h, j), max(h, j)) for j in rng.choice(n, n // 3, replace=False) if j != h}
    A = np.zeros((n, n))
    for i, j in edges:
        w = rng.uniform(0.5, 1.5)
        A[i, j] = A[j, i] = -w
    A[np.arange(n), np.arange(n)] = -A.sum(1) + 0.1
    return A


def dense_to_csr(A):
    rows, cols = np.nonzero(A)
    rp = np.zeros(A.shape[0] + 1, np.int32)
    np.add.at(rp, rows + 1, 1)
    return np.cumsum(rp).astype(np.int32), cols.astype(np.int32), A[rows, cols]


@pytest.mark.parametrize("precision,block", [(fem.PRECISION_FP64, 0), (fem.PRECISION_MIXED, 0),
                                             (fem.PRECISION_MIXED, 3)])
def test_cg_on_uneven_rows_matches_oracle(cuda_ctx, precision, block):
    """The iteration SpMVs read sliced-ELL copies (32 rows, or 32 block rows,
    per slice, padded to the slice's longest row): rows of 2 to ~340 entries,
    a last slice cut short (1001 rows, or 3 x 1001 scalar rows for the 3x3
    blocks), FP64 CG and mixed precision against the oracle's solution."""
    L = hub_laplacian(1001, hubs=[5, 500, 999], seed=3)
    A = np.kron(L, np.array([[4.0, 1.0, 0.5], [1.0, 3.0, 0.2], [0.5, 0.2, 2.0]])) if block == 3 else L
    rp, cols, vals = dense_to_csr(A)
    b = np.random.default_rng(4).standard_normal(A.shape[0])
    dev = lambda a: torch.as_tensor(a, device="cuda")
    x = torch.zeros(A.shape[0], dtype=torch.float64, device="cuda")
    opt = fem.solver_options(rtol=1e-10, max_iter=20000, precision=precision)
    opt.block_size = block
    info = fem.cg_solve_csr(cuda_ctx, dev(rp), dev(cols), dev(vals), dev(b), x, options=opt)
    assert info.status == 0 and info.relres < 1e-10
    x_ref, _, _ = O.pcg_jacobi(rp, cols, vals, b, rtol=1e-13, max_iter=50000)
    assert np.linalg.norm(x.cpu().numpy() - x_ref) / np.linalg.norm(x_ref) < 1e-8
