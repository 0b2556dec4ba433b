"""The learned preconditioner on an unstructured mesh of the reference:
meshes/msh/circle_cut.msh (the poisson module's circle test, fixture
tests/golden/poisson_circle_2d.npz) with the reference's penalty Dirichlet
conditions.  The level hierarchy is algebraic (learned.AlgebraicHierarchy:
smoothed aggregation on the matrix), not the structured grid's.

  * the network's forward pass and gradient on that hierarchy against the
    numpy oracle (same tolerances as on the structured grid);
  * the solve through the linear system with precond = learned
    (afem_ls_set_learned_preconditioner + afem_ls_solve, penalty rows out of
    the stop test): the reference's check file within its 1e-4, and the same
    solution as Jacobi CG to 1e-8;
  * a few training steps on solver-generated pairs lower the loss, and the
    trained network still solves to the check file.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

import golden_cases as G
from arcanefem_gb300 import fem, learned, meshgen
from oracle import mpnn_oracle as MO

pytestmark = pytest.mark.gpu

NAME = "poisson_circle_2d"


def circle_system(ctx):
    spec = G.CASES[NAME]
    d = G.load(NAME)
    mesh = meshgen.Mesh(2, d["coords"], d["cells"])
    f = fem.BSRFormat(ctx, fem.Mesh.from_host(2, mesh.coords, mesh.cells))
    f.initialize(1)
    f.compute_sparsity()
    f.assemble_poisson()
    ls = fem.DoFLinearSystem(ctx, mesh.nb_node)
    f.to_linear_system(ls)
    f.rhs_constant_source(spec["f"], ls.rhs_variable())
    for g, v in spec["dirichlet"]:
        ls.apply_dirichlet_penalty(torch.as_tensor(d["group__" + g], device="cuda"), 1, 0, v, spec["penalty"])
    ls.apply_matrix_transformation()
    ls.apply_rhs_transformation()
    return d, f, ls


def test_algebraic_hierarchy_forward_and_gradient_match_oracle(cuda_ctx):
    d, f, ls = circle_system(cuda_ctx)
    rp, cols, vals = f.row_ptr, f.cols, f.values
    hier = learned.AlgebraicHierarchy(rp, cols, vals, min_coarse=16)
    assert hier.levels >= 3 and hier.rows[-1] < hier.rows[0]
    layers = min(3, hier.levels)
    net = learned.MPNN(cuda_ctx, hier, layers=layers, max_batch=2)
    try:
        params = net.init_params(seed=3, head_scale=0.1, edge_scale=0.3)
        net.set_params(params)
        net.set_operator(rp, cols, vals)
        n = rp.numel() - 1
        A = sp.csr_matrix((vals.cpu().numpy(), cols.cpu().numpy(), rp.cpu().numpy()), shape=(n, n))
        onet = MO.Net(A, hier.host_graph, hier.host_restr, hier.host_prol, layers=net.layers, bf16_round=True,
                      fact_rows=MO.FACT_ROWS, exact_rows=MO.EXACT_ROWS)
        rng = np.random.default_rng(1)
        free = (A.diagonal() < 1e20).astype(np.float64)   # errors on the free nodes only
        E = rng.standard_normal((2, n)) * free
        R = np.stack([A @ e for e in E])
        Rt = torch.as_tensor(R, dtype=torch.float32, device="cuda").contiguous()
        Et = torch.as_tensor(E, dtype=torch.float32, device="cuda").contiguous()
        z = net.forward(Rt).cpu().numpy().reshape(2, n)
        p64 = net.get_params().astype(np.float64)
        zo = np.stack([onet.forward(p64, r) for r in R])
        for k in range(2):
            assert np.linalg.norm(z[k] - zo[k]) <= 1e-2 * np.linalg.norm(zo[k])
        g, loss = net.gradients(Rt, Et)
        lo, go = onet.loss_and_grad(p64, [r.astype(np.float32).astype(np.float64) for r in R],
                                    [e.astype(np.float32).astype(np.float64) for e in E])
        g = g.cpu().numpy()
        assert abs(loss - lo) <= 1e-2 * lo
        assert np.dot(g, go) / (np.linalg.norm(g) * np.linalg.norm(go)) > 0.99
    finally:
        net.close()


def test_learned_solve_through_the_linear_system_matches_the_check_file(cuda_ctx):
    spec = G.CASES[NAME]
    d, f, ls = circle_system(cuda_ctx)
    rp, cols, vals = f.row_ptr, f.cols, f.values
    hier = learned.AlgebraicHierarchy(rp, cols, vals, min_coarse=16)
    net = learned.MPNN(cuda_ctx, hier, layers=min(6, hier.levels), max_batch=8)
    try:
        net.set_params(net.init_params(seed=7))
        ls.set_learned_preconditioner(net)
        opt = fem.solver_options(rtol=1e-12, max_iter=500, precond=fem.PRECOND_LEARNED, skip_forced_rows=True)
        info = ls.solve(opt)
        assert info.status == 0 and info.relres < 1e-12, (info.iterations, info.relres)
        u = ls.solution_variable().cpu().numpy()
        err = G.compare(NAME, u, d)
        assert err < spec["eps"], err
        # the same solution as Jacobi CG
        x = torch.zeros_like(ls.rhs_variable())
        fem.cg_solve_csr(cuda_ctx, rp, cols, vals, ls.rhs_variable(), x, ls.get_forced_info(),
                         fem.solver_options(rtol=1e-12, max_iter=20000, skip_forced_rows=True))
        xc = x.cpu().numpy()
        assert np.linalg.norm(u - xc) <= 1e-8 * np.linalg.norm(xc)
        it_untrained = info.iterations
        # a few training steps on pairs the solver generates: errors of restarted Jacobi-CG iterates
        n = rp.numel() - 1
        forced = ls.get_forced_info().clone()
        Rs, Es = [], []
        rng = np.random.default_rng(5)
        for s in range(4):
            b = torch.as_tensor(rng.standard_normal(n), device="cuda") * (1 - forced.double())
            xs = torch.zeros_like(b)
            fem.cg_solve_csr(cuda_ctx, rp, cols, vals, b, xs, None, fem.solver_options(rtol=1e-12, max_iter=20000))
            xk = torch.zeros_like(b)
            for k in range(4):
                e = xs - xk
                y = torch.empty_like(e)
                fem.spmv_csr(cuda_ctx, rp, cols, vals, e, y)
                Rs.append(y.float())
                Es.append(e.float())
                try:
                    fem.cg_solve_csr(cuda_ctx, rp, cols, vals, b, xk, None, fem.solver_options(rtol=1e-300,
                                                                                               max_iter=3))
                except fem.AfemError as ex:
                    assert ex.status == 3
        R = torch.stack(Rs).contiguous()
        E = torch.stack(Es).contiguous()
        hist = learned.train(net, R, E, epochs=3, batch=8, lr=1e-3)
        assert np.isfinite(hist).all() and hist[-1] < hist[0]
        ls.solution_variable().zero_()
        info2 = ls.solve(opt)
        assert info2.status == 0 and G.compare(NAME, ls.solution_variable().cpu().numpy(), d) < spec["eps"]
        assert info2.iterations <= 2 * it_untrained
    finally:
        ls.set_learned_preconditioner(None)
        net.close()
