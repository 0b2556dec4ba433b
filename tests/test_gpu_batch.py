"""Batched persistent assembly + solve on the GPU against the CPU oracle:
assembled and eliminated matrices per instance, lumped bump sources,
solutions to the FP64 residual target, determinism, the autotuner and its
cache, and failure detection of a team barrier that never completes."""
import json

import numpy as np
import pytest
import torch

from arcanefem_gb300 import batch as B
from arcanefem_gb300 import fem
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SIZES = [8, 12, 16, 20, 24, 32, 5, 40]


def oracle_instance(bt, i):
    m = bt.meshes[i]
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    rp, cols = O.sparsity(m.nb_node, m.cells)
    v = O.assemble(O.POISSON_TRI3, m.coords, m.cells, ptr, nc, rp, cols)
    ei, ev = np.zeros(m.nb_node, np.uint8), np.zeros(m.nb_node)
    fi, fv = np.zeros(m.nb_node, np.uint8), np.zeros(m.nb_node)
    O.dirichlet_elimination(m.groups["boundary"], 1, 0, 0.0, 2, ei, ev)
    rhs = np.zeros(m.nb_node)
    O.apply_transformations(rp, cols, v, rhs, fi, fv, ei, ev)
    # lumped area and the bump sources (FP32 evaluation, as the kernel)
    mass = np.zeros(m.nb_node)
    P = m.coords[m.cells][:, :, :2]
    area = 0.5 * np.abs((P[:, 1, 0] - P[:, 0, 0]) * (P[:, 2, 1] - P[:, 0, 1])
                        - (P[:, 1, 1] - P[:, 0, 1]) * (P[:, 2, 0] - P[:, 0, 0]))
    for k in range(3):
        np.add.at(mass, m.cells[:, k], area / 3.0)
    src = bt.sources[i].cpu().numpy()
    px, py = m.coords[:, 0].astype(np.float32), m.coords[:, 1].astype(np.float32)
    b = np.zeros((m.nb_node, 4))
    for j in range(4):
        f = np.zeros(m.nb_node, np.float32)
        for a, cx, cy, w in src[j]:
            f += a * np.exp(-((px - cx) ** 2 + (py - cy) ** 2) / (2 * w * w))
        b[:, j] = mass * f.astype(np.float64)
    b[m.groups["boundary"]] = 0.0
    return rp, cols, v, b


@pytest.fixture(scope="module")
def small_batch():
    ctx = fem.Context()
    bt = B.Batch(ctx, SIZES, seed=3, jitter=0.2)
    yield ctx, bt
    bt.close()


def test_batch_assembly_rhs_and_solutions_match_oracle(small_batch):
    ctx, bt = small_batch
    rtol = 1e-10
    res, ms = bt.solve(fem.solver_options(rtol=rtol, inner_rtol=0.1, max_iter=20000))
    assert ms > 0
    for i, n in enumerate(SIZES):
        rp, cols, v, b = oracle_instance(bt, i)
        assert np.array_equal(bt.fmts[i].row_ptr.cpu().numpy(), rp)
        vg = bt.fmts[i].values.cpu().numpy()
        # assembled + eliminated matrix: 1e-12 relative per entry (same arithmetic: exact in practice)
        assert np.all(np.abs(vg - v) <= 1e-12 * np.maximum(np.abs(v), 1e-300)), i
        bg = bt.rhs[i].cpu().numpy()
        assert np.abs(bg - b).max() <= 1e-6 * np.abs(b).max(), i
        x = bt.x[i].cpu().numpy()
        r = res[i]
        assert r.status == 0 and r.refinements >= 1
        for j in range(4):
            ax = O.spmv(rp, cols, v, x[:, j])
            rel = np.linalg.norm(bg[:, j] - ax) / np.linalg.norm(bg[:, j])
            assert rel <= rtol * 1.01 and abs(rel - r.relres[j]) <= 1e-3 * rtol + 1e-15, (i, j, rel, r.relres[j])
            xo, _, _ = O.pcg_jacobi(rp, cols, v, bg[:, j], rtol=1e-13)
            assert np.linalg.norm(x[:, j] - xo) <= 1e-7 * np.linalg.norm(xo), (i, j)


def test_batch_is_deterministic_and_reusable(small_batch):
    ctx, bt = small_batch
    opt = fem.solver_options(rtol=1e-8, inner_rtol=0.1, max_iter=20000)
    bt.solve(opt)
    x1 = [x.clone() for x in bt.x]
    res, _ = bt.solve(opt)
    for a, b in zip(x1, bt.x):
        assert torch.equal(a, b)
    assert all(r.status == 0 and max(r.relres) <= 1e-8 for r in res)


def test_team_partition_covers_the_grid(small_batch):
    ctx, bt = small_batch
    for block, bps in ((128, 1), (256, 2), (512, 1)):
        bt.set_config(block, bps, 3.0)
        cfg, grid = bt.config()
        spans = sorted(bt.team(i) for i in range(len(SIZES)))
        assert spans[0][0] == 0 and all(s[1] >= 1 for s in spans)
        assert all(spans[k][0] + spans[k][1] == spans[k + 1][0] for k in range(len(spans) - 1))
        assert spans[-1][0] + spans[-1][1] == grid
        # larger instances never get fewer CTAs than smaller ones
        order = np.argsort(SIZES)
        counts = [bt.team(int(i))[1] for i in order]
        assert counts == sorted(counts)
        res, _ = bt.solve(fem.solver_options(rtol=1e-8, inner_rtol=0.1, max_iter=20000))
        assert all(r.status == 0 for r in res)
    bt.set_config(256, 1, 3.0)


def test_autotuner_picks_and_caches(small_batch, tmp_path):
    ctx, bt = small_batch
    cache = str(tmp_path / "tune.json")
    cands = [(128, 1, 3.0), (256, 1, 3.0), (256, 1, 2.0)]
    out = bt.autotune(candidates=cands, reps=1, cache=cache)
    assert not out["cached"] and len(out["times_ms"]) == 3 and min(out["times_ms"]) > 0
    best = int(np.argmin(out["times_ms"]))
    assert out["config"]["block"] == cands[best][0]
    table = json.load(open(cache))
    assert len(table) == 1
    again = bt.autotune(candidates=cands, reps=1, cache=cache)
    assert again["cached"] and again["config"] == out["config"]
    cfg, _ = bt.config()
    assert cfg.block == out["config"]["block"]
    bt.set_weights(None)


def test_rebalance_from_measured_finish_times(small_batch):
    ctx, bt = small_batch
    bt.set_config(256, 1, 3.0)
    ms0 = bt.solve()[1]
    ms, w = bt.rebalance(rounds=2)
    assert ms <= ms0 * 1.25   # the kept split is the fastest seen (timing noise aside)
    if w is not None:
        assert len(w) == len(SIZES) and all(v > 0 for v in w)
    res, _ = bt.solve()
    assert all(r.status == 0 and r.finish_ms > 0 for r in res)
    bt.set_weights(None)


def test_barrier_wait_runs_out_and_context_survives(small_batch):
    """A CTA that never arrives: its teammates' bounded waits end with
    AFEM_ERR_TIMEOUT; the next batch solve on the same context succeeds."""
    ctx, bt = small_batch
    bt.set_config(256, 1, 3.0)
    big = int(np.argmax(SIZES))
    cta0, ncta = bt.team(big)
    assert ncta >= 2
    status = bt.failure_test(cta0 + 1, spin_limit=200000)
    assert status == 5   # AFEM_ERR_TIMEOUT
    res, _ = bt.solve(fem.solver_options(rtol=1e-8, inner_rtol=0.1, max_iter=20000))
    assert all(r.status == 0 for r in res)
