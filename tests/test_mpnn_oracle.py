"""The CPU oracle of the learned preconditioner: its analytic gradient against
central finite differences (float64) on a small hierarchy, symmetry and
positivity of the V-cycle, the conditioning of its untrained form, and the
hierarchy's transfers."""
import numpy as np
import pytest
import scipy.sparse as sp

from arcanefem_gb300 import learned, meshgen
from oracle import mpnn_oracle as MO
from oracle import oracle as O


def small_problem(n=8, levels=3, seed=0, dirichlet=True):
    m = meshgen.unit_square_tri(n, jitter=0.2, seed=seed)
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    rp, cols = O.sparsity(m.nb_node, m.cells)
    k = np.exp(np.random.default_rng(seed).standard_normal(m.nb_cell))
    v = O.assemble(O.POISSON_TRI3, m.coords, m.cells, ptr, nc, rp, cols, cell_coeff=k)
    ei, ev = np.zeros(m.nb_node, np.uint8), np.zeros(m.nb_node)
    fi, fv = np.zeros(m.nb_node, np.uint8), np.zeros(m.nb_node)
    O.dirichlet_elimination(m.groups["boundary"], 1, 0, 0.0, 2, ei, ev)
    rhs = np.zeros(m.nb_node)
    O.apply_transformations(rp, cols, v, rhs, fi, fv, ei, ev)
    A = sp.csr_matrix((v, cols, rp), shape=(m.nb_node, m.nb_node))
    sizes = [(n >> l) + 1 for l in range(levels)]
    graphs = [None] + [learned.grid_graph(s) for s in sizes[1:]]
    R = [learned.restriction(sizes[l]) for l in range(levels - 1)]
    if dirichlet:
        P = [learned.masked_prolongation(R[l], sizes[l]) for l in range(levels - 1)]
    else:
        P = [learned.prolongation(r) for r in R]
    return A, graphs, R, P, m


def symmetric_elimination(A, m):
    """The eliminated matrix without the reference's kept column 0
    (CsrDoFLinearSystemImpl.cc:111 tests column_index > 0): identity rows and
    zero columns on every Dirichlet node, so A is exactly symmetric."""
    keep = np.ones(A.shape[0])
    keep[m.groups["boundary"]] = 0
    return sp.csr_matrix(sp.diags(keep) @ A @ sp.diags(keep) + sp.diags(1 - keep))


def operator_matrix(net, c, n):
    return np.stack([net.apply(c, np.eye(n)[i])[0] for i in range(n)], 1)


@pytest.mark.parametrize("layers", [3, 2])
def test_oracle_gradient_matches_finite_differences(layers):
    A, graphs, R, P, m = small_problem()
    # the energy loss's gradient -2 A (e - z) and the V-cycle adjoint assume
    # a symmetric A; the reference's row-column elimination leaves column 0
    # in place, so drop that column here
    A = symmetric_elimination(A, m)
    net = MO.Net(A, graphs, R, P, layers=layers, fact_rows=MO.FACT_ROWS)
    rng = np.random.default_rng(1)
    params = learned.init_params(net.NL, net.L, seed=3, head_scale=0.2, nfact=net.nfact).astype(np.float64)
    params[2 * 64:3 * 64] = 0.1                       # biases away from zero
    assert params.size == MO.param_count(net.NL, net.L, net.nfact)
    edges = MO.param_count(net.NL, net.L)
    params[edges:] = rng.normal(0, 0.3, params.size - edges)   # edge heads away from zero
    c = net.features(params)
    # every level is factored here, and some level's theta comes from its
    # bound, so that the gradient through the maximal row is checked too
    assert net.fact == list(range(net.L))
    if layers == 3:
        assert min(c["f"][l]["theta"] for l in net.fact) < 1.0
    rs = [A @ rng.standard_normal(A.shape[0]) for _ in range(2)]
    es = [rng.standard_normal(A.shape[0]) for _ in range(2)]
    loss, g = net.loss_and_grad(params, rs, es)
    heads = edges - net.L * 65
    idx = np.concatenate([rng.choice(g.size, 40, replace=False),
                          [0, 1, 64, 128, 200, heads, heads + 64, edges - 66, edges - 1],
                          edges + rng.choice(params.size - edges, 30, replace=False)])
    eps = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += eps
        p2[i] -= eps
        fd = (net.loss_and_grad(p1, rs, es)[0] - net.loss_and_grad(p2, rs, es)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-4 * abs(fd) + 1e-8, (i, fd, g[i])


def test_preconditioner_is_symmetric_positive_definite():
    A, graphs, R, P, m = small_problem(n=16, levels=4)
    A = symmetric_elimination(A, m)
    net = MO.Net(A, graphs, R, P, layers=2, fact_rows=MO.FACT_ROWS)
    params = learned.init_params(net.NL, net.L, seed=1, head_scale=0.3, nfact=net.nfact).astype(np.float64)
    edges = MO.param_count(net.NL, net.L)
    params[edges:] = np.random.default_rng(2).normal(0, 1.0, params.size - edges)   # strong edge heads
    c = net.features(params)
    d = c["d"]
    assert max(np.abs(np.log(d[l][d[l] > 0] / net.base[l][d[l] > 0])).max() for l in range(net.L)) > 1e-2
    assert max(abs(c["f"][l]["m"]).max() for l in net.fact if c["f"][l]["m"].size) > 0.5
    M = operator_matrix(net, c, A.shape[0])
    assert np.abs(M - M.T).max() <= 1e-12 * np.abs(M).max()
    assert np.linalg.eigvalsh(0.5 * (M + M.T)).min() > 0
    for Al in net.Al:
        assert abs(Al - Al.T).max() <= 1e-12 * abs(Al).max()


def _pcg_spectrum(A, M):
    Ls = np.linalg.cholesky(0.5 * (M + M.T))
    ev = np.linalg.eigvalsh(Ls.T @ A.toarray() @ Ls)
    return ev.min(), ev.max()


def test_vcycle_conditions_far_better_than_jacobi():
    """With zero heads the operator is one V(1,1)-cycle with l1-Jacobi
    smoothing on the Galerkin hierarchy: its spectrum on the
    variable-coefficient Laplacian lies in (0, ~1] and its condition number
    is a small constant, far below Jacobi's."""
    A, graphs, R, P, m = small_problem(n=32, levels=5)
    A = symmetric_elimination(A, m)
    net = MO.Net(A, graphs, R, P, fact_rows=MO.FACT_ROWS)
    c = net.features(np.zeros(MO.param_count(net.NL, net.L, net.nfact)))
    d = c["d"]
    assert np.allclose(d[0], MO.THETA * 2 / np.asarray(abs(A).sum(axis=1)).ravel())
    # zero edge heads: the factored smoothers are exactly the diagonal ones
    assert all(c["f"][l]["theta"] == 1.0 for l in net.fact)
    n = A.shape[0]
    lo, hi = _pcg_spectrum(A, operator_matrix(net, c, n))
    jlo, jhi = _pcg_spectrum(A, np.diag(1.0 / net.d))
    # the V-cycle with exact coarsest solves is an A-contraction (spectrum in
    # (0, 1]); the coarsest level here is one l1-Jacobi step, so allow a little
    assert 0 < lo and hi <= 1.05, (lo, hi)
    assert hi / lo < 4, (lo, hi)
    assert (hi / lo) * 50 < jhi / jlo, (hi / lo, jhi / jlo)


def test_hierarchy_operators():
    n = 16
    R = learned.restriction(n + 1)
    assert R.shape == ((n // 2 + 1) ** 2, (n + 1) ** 2)
    # full weighting preserves constants in the interior
    ones = np.ones((n + 1) ** 2)
    c = (R @ ones).reshape(n // 2 + 1, n // 2 + 1)
    assert np.allclose(c[1:-1, 1:-1], 1.0)
    P = learned.prolongation(R)
    assert abs(P - 4.0 * R.T).max() == 0
    # bilinear prolongation reproduces linear functions on the fine grid
    xc = np.tile(np.linspace(0, 1, n // 2 + 1), n // 2 + 1)
    xf = np.tile(np.linspace(0, 1, n + 1), n + 1)
    assert np.allclose((P @ xc).reshape(n + 1, n + 1)[1:-1, 1:-1], xf.reshape(n + 1, n + 1)[1:-1, 1:-1])
    # the masked form vanishes on the fine boundary and ignores coarse boundary values
    Pm = learned.masked_prolongation(R, n + 1)
    y = (Pm @ np.random.default_rng(0).standard_normal((n // 2 + 1) ** 2)).reshape(n + 1, n + 1)
    assert np.all(y[0] == 0) and np.all(y[-1] == 0) and np.all(y[:, 0] == 0) and np.all(y[:, -1] == 0)
    G = learned.grid_graph(5)
    # 8-neighbour graph of a 5 x 5 grid: 2 x (20 horizontal + 20 vertical + 32 diagonal) directed edges
    assert abs(G - G.T).max() == 0 and G.nnz == 144


def test_exact_coarse_level_gradient_and_spd():
    """With an exact level (the first level below the finest of at most 320
    rows: here level 1, 289 rows), the V-cycle stops there and solves it with
    the inverse of its nonzero rows' block; the gradient (no parameter on that
    level) still matches central finite differences, and M stays SPD."""
    A, graphs, R, P, m = small_problem(n=32, levels=5)
    A = symmetric_elimination(A, m)
    net = MO.Net(A, graphs, R, P, layers=3, fact_rows=MO.FACT_ROWS, exact_rows=MO.EXACT_ROWS)
    assert net.ex == 1 and net.Lv == 2 and net.fact == [0]
    rng = np.random.default_rng(1)
    params = learned.init_params(net.NL, net.L, seed=3, head_scale=0.2, nfact=net.nfact).astype(np.float64)
    params[2 * 64:3 * 64] = 0.1
    edges = MO.param_count(net.NL, net.L)
    params[edges:] = rng.normal(0, 0.3, params.size - edges)
    n = A.shape[0]
    es = [rng.standard_normal(n) for _ in range(2)]
    rs = [A @ e for e in es]
    loss, g = net.loss_and_grad(params, rs, es)
    idx = np.concatenate([rng.choice(edges, 30, replace=False), edges + np.arange(params.size - edges)])
    eps = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += eps
        p2[i] -= eps
        fd = (net.loss_and_grad(p1, rs, es)[0] - net.loss_and_grad(p2, rs, es)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-4 * abs(fd) + 1e-8, (i, fd, g[i])
    c = net.features(params)
    M = operator_matrix(net, c, n)
    assert np.abs(M - M.T).max() <= 1e-12 * np.abs(M).max()
    assert np.linalg.eigvalsh(0.5 * (M + M.T)).min() > 0


@pytest.mark.parametrize("sizes", [
    [263169, 66049, 16641, 4225, 1089, 289, 81, 25, 9],   # 513^2, 9 levels (the bench)
    [66049, 16641, 4225, 1089, 289, 81, 25, 9],           # 257^2 (the learned test)
    [4225, 1089, 289, 81],
    [5000, 3000, 2100, 2048, 400, 321, 320, 12],          # the thresholds themselves
    [700, 330, 200],
    [200, 90],
    [9000, 4000],                                          # no exact level
])
def test_level_rules_agree_with_the_oracle(sizes):
    """The library's host rules for the exactly solved level, the factored
    levels and the parameter count (arcanefem_gb300/learned.py, mirrored by the
    device code) are the oracle's: the parameter vector one side packs is the
    one the other unpacks."""
    from arcanefem_gb300 import learned
    assert learned.FACT_ROWS == MO.FACT_ROWS and learned.EXACT_ROWS == MO.EXACT_ROWS
    ex = MO.exact_level(sizes)
    assert learned.exact_level(sizes) == ex
    fl = MO.fact_levels(sizes, MO.FACT_ROWS, ex)
    assert learned.fact_levels(sizes) == fl
    assert 0 in fl and (ex is None or all(l < ex for l in fl))
    for layers in (1, 3, 6):
        assert learned.param_count(layers, len(sizes), len(fl)) == MO.param_count(layers, len(sizes), len(fl))

