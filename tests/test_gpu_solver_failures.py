"""Failure statuses of every solver, made on the host (no device fault):

  * a non-SPD matrix (negated diagonal)            -> AFEM_ERR_BREAKDOWN
  * a NaN in the right-hand side                   -> AFEM_ERR_BREAKDOWN
  * max_iter reached                               -> AFEM_ERR_NOT_CONVERGED, with
    the last iterate in the solution argument and its true residual in the info

for afem_cg_solve_csr (FP64 and mixed precision), afem_ls_solve,
afem_fcg_solve (learned preconditioner) and afem_batch_solve (per instance).
The reference maps a solver library's error codes to exceptions
(femutils/HypreDoFLinearSystem.cc:86-111); here the status code comes back
and the Python layer raises AfemError carrying the SolveInfo.  After each
failure the context is used again for a good solve.
"""
import numpy as np
import pytest
import torch

from arcanefem_gb300 import batch as B
from arcanefem_gb300 import fem, learned, meshgen
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NOT_CONVERGED, BREAKDOWN = 3, 4


def poisson(ctx, n=8):
    """Transformed 3D Poisson system (row-column elimination on the x faces)."""
    m = meshgen.unit_cube_tet(n, seed=5)
    f = fem.BSRFormat(ctx, fem.Mesh.from_host(3, m.coords, m.cells))
    f.initialize(1)
    f.compute_sparsity()
    f.assemble_poisson()
    ls = fem.DoFLinearSystem(ctx, m.nb_node)
    f.to_linear_system(ls)
    f.rhs_constant_source(1.0, ls.rhs_variable())
    ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, torch.as_tensor(m.groups["x_faces"], device="cuda"), 1,
                                   0, 0.0)
    ls.apply_matrix_transformation()
    ls.apply_rhs_transformation()
    rp, cols, vals = f.row_ptr, f.cols, f.values
    return f, ls, rp, cols, vals, ls.rhs_variable().clone()


def true_relres(rp, cols, vals, b, x):
    r = b.cpu().numpy() - O.spmv(rp.cpu().numpy(), cols.cpu().numpy(), vals.cpu().numpy(), x.cpu().numpy())
    return float(np.linalg.norm(r) / np.linalg.norm(b.cpu().numpy()))


def negated_diagonal(rp, cols, vals):
    v = vals.clone()
    rpc, cc = rp.cpu().numpy(), cols.cpu().numpy()
    row = np.repeat(np.arange(rpc.size - 1), np.diff(rpc))
    diag = torch.as_tensor(np.flatnonzero(cc == row), device=v.device)
    v[diag] = -v[diag]
    return v


PRECISIONS = [fem.PRECISION_FP64, fem.PRECISION_MIXED]


@pytest.mark.parametrize("precision", PRECISIONS)
def test_cg_max_iter_gives_not_converged_and_the_last_iterate(cuda_ctx, precision):
    _, _, rp, cols, vals, b = poisson(cuda_ctx)
    x = torch.zeros_like(b)
    with pytest.raises(fem.AfemError) as e:
        fem.cg_solve_csr(cuda_ctx, rp, cols, vals, b, x,
                         options=fem.solver_options(rtol=1e-12, max_iter=5, precision=precision))
    assert e.value.status == NOT_CONVERGED
    info = e.value.info
    assert info.status == NOT_CONVERGED and 0 < info.iterations <= 5
    res = true_relres(rp, cols, vals, b, x)
    assert 1e-12 < res < 1.0                     # progress, not convergence
    assert abs(res - info.relres) <= 1e-6 * res   # the info's residual is that of the returned iterate
    # the context is still good
    x.zero_()
    ok = fem.cg_solve_csr(cuda_ctx, rp, cols, vals, b, x, options=fem.solver_options(rtol=1e-10, max_iter=5000,
                                                                                     precision=precision))
    assert ok.status == 0 and true_relres(rp, cols, vals, b, x) < 1e-10


@pytest.mark.parametrize("precond", [fem.PRECOND_JACOBI, fem.PRECOND_NONE])
@pytest.mark.parametrize("precision", PRECISIONS)
def test_cg_non_spd_matrix_breaks_down(cuda_ctx, precision, precond):
    _, _, rp, cols, vals, b = poisson(cuda_ctx)
    bad = negated_diagonal(rp, cols, vals)
    x = torch.zeros_like(b)
    with pytest.raises(fem.AfemError) as e:
        fem.cg_solve_csr(cuda_ctx, rp, cols, bad, b, x,
                         options=fem.solver_options(rtol=1e-10, max_iter=500, precision=precision, precond=precond))
    assert e.value.status == BREAKDOWN and e.value.info.status == BREAKDOWN
    assert "breakdown" in str(e.value).lower()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_cg_nan_rhs_breaks_down(cuda_ctx, precision):
    _, _, rp, cols, vals, b = poisson(cuda_ctx)
    b = b.clone()
    b[len(b) // 2] = float("nan")
    x = torch.zeros_like(b)
    with pytest.raises(fem.AfemError) as e:
        fem.cg_solve_csr(cuda_ctx, rp, cols, vals, b, x, options=fem.solver_options(rtol=1e-10, max_iter=500,
                                                                                    precision=precision))
    assert e.value.status == BREAKDOWN


def test_linear_system_solve_statuses(cuda_ctx):
    f, ls, rp, cols, vals, b = poisson(cuda_ctx)
    with pytest.raises(fem.AfemError) as e:
        ls.solve(fem.solver_options(rtol=1e-12, max_iter=3))
    assert e.value.status == NOT_CONVERGED and e.value.info.iterations == 3
    assert abs(true_relres(rp, cols, vals, b, ls.solution_variable()) - e.value.info.relres) <= 1e-6
    # a non-SPD matrix behind the same linear system
    neg = negated_diagonal(rp, cols, vals)
    ls.set_csr_values(rp, cols, neg)
    ls.solution_variable().zero_()
    with pytest.raises(fem.AfemError) as e:
        ls.solve(fem.solver_options(rtol=1e-10, max_iter=500))
    assert e.value.status == BREAKDOWN
    ls.set_csr_values(rp, cols, vals)
    ls.solution_variable().zero_()
    assert ls.solve(fem.solver_options(rtol=1e-10, max_iter=5000)).status == 0


def test_learned_fcg_statuses(cuda_ctx):
    prob, hier, net = learned.setup(cuda_ctx, n=16, levels=3, layers=2, seed=1, max_batch=1)
    try:
        net.set_params(net.init_params(seed=2, head_scale=0.1))
        b = prob.rhs(np.random.default_rng(3))
        x = torch.zeros_like(b)
        with pytest.raises(fem.AfemError) as e:
            net.fcg(prob.row_ptr, prob.cols, prob.values, b, x, fem.solver_options(rtol=1e-14, max_iter=2))
        assert e.value.status == NOT_CONVERGED and e.value.info.iterations == 2
        assert 0.0 < true_relres(prob.row_ptr, prob.cols, prob.values, b, x) < 1.0
        x.zero_()
        bad = negated_diagonal(prob.row_ptr, prob.cols, prob.values)
        with pytest.raises(fem.AfemError) as e:
            net.fcg(prob.row_ptr, prob.cols, bad, b, x, fem.solver_options(rtol=1e-8, max_iter=100))
        assert e.value.status == BREAKDOWN
        x.zero_()
        assert net.fcg(prob.row_ptr, prob.cols, prob.values, b, x,
                       fem.solver_options(rtol=1e-8, max_iter=500)).relres < 1e-8
    finally:
        net.close()


def test_batch_reports_a_status_per_instance(cuda_ctx):
    bt = B.Batch(cuda_ctx, [8, 24], seed=1)
    try:
        with pytest.raises(fem.AfemError) as e:
            bt.solve(fem.solver_options(rtol=1e-12, inner_rtol=0.1, max_iter=2))
        res = e.value.results
        assert e.value.status == NOT_CONVERGED
        assert any(r.status == NOT_CONVERGED for r in res)
        assert all(r.status in (0, NOT_CONVERGED) for r in res)
        # the larger instance cannot reach 1e-12 in 30 cycles of 2 iterations
        assert res[1].status == NOT_CONVERGED and max(res[1].relres) > 1e-12
        res2, _ = bt.solve(fem.solver_options(rtol=1e-8, inner_rtol=0.1, max_iter=5000))
        assert all(r.status == 0 and max(r.relres) <= 1e-8 for r in res2)
    finally:
        bt.close()
