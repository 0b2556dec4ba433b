"""Learned preconditioner on the GPU: smoother weights, V-cycle forward and
gradients against the CPU oracle, training reduces the loss on held-out
pairs, and what the trained network gains in flexible CG over the same
V-cycle untrained (the method without it) and over Jacobi CG."""
import numpy as np
import pytest
import scipy.sparse as sp
import torch

from arcanefem_gb300 import fem, learned
from oracle import mpnn_oracle as MO

pytestmark = pytest.mark.gpu


def oracle_net(prob, hier, layers):
    rp = prob.row_ptr.cpu().numpy()
    cols = prob.cols.cpu().numpy()
    vals = prob.values.cpu().numpy()
    A = sp.csr_matrix((vals, cols, rp), shape=(rp.size - 1, rp.size - 1))
    graphs = [None] + [learned.grid_graph(s) for s in hier.sizes[1:]]
    R = [learned.restriction(hier.sizes[l]) for l in range(hier.levels - 1)]
    P = [learned.masked_prolongation(R[l], hier.sizes[l]) for l in range(hier.levels - 1)]
    return MO.Net(A, graphs, R, P, layers=layers, bf16_round=True, fact_rows=MO.FACT_ROWS,
                  exact_rows=MO.EXACT_ROWS)


def test_zero_heads_give_l1_jacobi_vcycle(cuda_ctx):
    """Zero parameters: every smoother weight is 0.8 of its l1 cap (the caps
    come from the Galerkin operators the library computes), and one
    application is the plain V-cycle of the oracle."""
    prob, hier, net = learned.setup(cuda_ctx, n=32, levels=4, layers=2, seed=2, max_batch=1)
    net.set_params(np.zeros(net.nparam, np.float32))
    onet = oracle_net(prob, hier, 2)
    for l in range(hier.levels):
        d = net.scalings(l).cpu().numpy()
        assert np.allclose(d, MO.THETA * onet.base[l], rtol=1e-5, atol=0), l
    e = torch.as_tensor(np.random.default_rng(4).standard_normal(prob.mesh.nb_node), device="cuda") * prob.interior
    r = prob.apply(e).float().contiguous()
    z = net.forward(r).cpu().numpy()
    zo = onet.forward(np.zeros(net.nparam), r.cpu().numpy().astype(np.float64))
    assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < 1e-5
    net.close()


@pytest.mark.parametrize("layers", [5, 3])
def test_forward_and_gradients_match_oracle(cuda_ctx, layers):
    prob, hier, net = learned.setup(cuda_ctx, n=32, levels=5, layers=layers, seed=5, max_batch=2)
    rng = np.random.default_rng(0)
    params = net.init_params(seed=9, head_scale=0.1, edge_scale=0.3)
    params[2 * 64:3 * 64] = 0.05
    net.set_params(params)
    n = prob.mesh.nb_node
    e = torch.as_tensor(rng.standard_normal((2, n)), device="cuda") * prob.interior
    r = torch.stack([prob.apply(e[0].contiguous()), prob.apply(e[1].contiguous())])
    R, E = r.float().contiguous(), e.float().contiguous()
    z = net.forward(R).cpu().numpy()
    g, loss = net.gradients(R, E)
    g = g.cpu().numpy()
    onet = oracle_net(prob, hier, layers)
    p64 = net.get_params().astype(np.float64)
    rs = [R[i].cpu().numpy().astype(np.float64) for i in range(2)]
    es = [E[i].cpu().numpy().astype(np.float64) for i in range(2)]
    zo = np.stack([onet.forward(p64, rs[i]) for i in range(2)])
    assert np.linalg.norm(z - zo) / np.linalg.norm(zo) < 1e-2
    lo, go = onet.loss_and_grad(p64, rs, es)
    assert abs(loss - lo) / lo < 1e-2
    cos = float(np.dot(g, go) / (np.linalg.norm(g) * np.linalg.norm(go)))
    rel = float(np.linalg.norm(g - go) / np.linalg.norm(go))
    assert cos > 0.998 and rel < 6e-2, (cos, rel)
    net.close()


def test_training_and_learned_fcg(cuda_ctx):
    prob, hier, net = learned.setup(cuda_ctx, n=256, levels=8, layers=6, seed=3, max_batch=16)
    R, E = learned.make_training_pairs(prob, count=768, solves=12, every=20, seed=4)
    Rv, Ev = learned.make_training_pairs(prob, count=32, solves=2, every=20, seed=40)   # held out

    def held_out_loss():
        return np.mean([net.gradients(Rv[i:i + 16], Ev[i:i + 16])[1] for i in range(0, 32, 16)])

    val_before = held_out_loss()
    b_val = prob.rhs(np.random.default_rng(98))
    held = [prob.rhs(np.random.default_rng(200 + k)) for k in range(3)]   # never seen by training or the gate

    def held_out_iterations():
        its = []
        for b in held:
            x = torch.zeros_like(b)
            info = net.fcg(prob.row_ptr, prob.cols, prob.values, b, x, fem.solver_options(rtol=1e-8, max_iter=2000))
            assert info.status == 0 and info.relres < 1e-8
            its.append(info.iterations)
        return its

    its_untrained = held_out_iterations()
    rep = learned.train_validated(net, prob, R, E, b_val, epochs=4, batch=16, lr=5e-3)
    hist = rep["loss"]
    assert hist[-1] < hist[0], hist
    val_after = held_out_loss()
    print(f"held-out energy loss {val_before:.4f} -> {val_after:.4f}")
    # what training gains over the same V-cycle untrained (l1-Jacobi smoothers,
    # the method without the network): a lower error-propagation energy on pairs
    # it never saw, and at least 15 % fewer FCG iterations on a held-out right-hand side
    assert val_after < val_before, (val_before, val_after)
    its_trained = held_out_iterations()
    print(f"held-out FCG iterations: untrained {its_untrained}, trained {its_trained}")
    assert sum(its_trained) <= 0.85 * sum(its_untrained), (its_untrained, its_trained)
    assert rep["iterations_trained"] < rep["iterations_untrained"], rep
    assert rep["kept"] == "trained"
    b = prob.rhs(np.random.default_rng(99))
    _, info_cg = prob.cg(b, rtol=1e-8)
    x = torch.zeros_like(b)
    info = net.fcg(prob.row_ptr, prob.cols, prob.values, b, x, fem.solver_options(rtol=1e-8, max_iter=2000))
    assert info.status == 0 and info.relres < 1e-8
    print(f"FCG untrained {rep['iterations_untrained']}, trained {rep['iterations_trained']} "
          f"(kept {rep['kept']}), test rhs {info.iterations}, Jacobi CG {info_cg.iterations}")
    # against plain Jacobi CG
    assert info.iterations * 10 < info_cg.iterations, (info.iterations, info_cg.iterations)
    # the solver's judgement keeps the better parameter set
    xv = torch.zeros_like(b_val)
    kept = net.fcg(prob.row_ptr, prob.cols, prob.values, b_val, xv, fem.solver_options(rtol=1e-8, max_iter=2000))
    assert kept.iterations == min(rep["iterations_untrained"], rep["iterations_trained"])
    # the device-side FCG graph is reused on a second solve with the same pointers
    x.zero_()
    info2 = net.fcg(prob.row_ptr, prob.cols, prob.values, b, x, fem.solver_options(rtol=1e-8, max_iter=2000))
    assert info2.iterations == info.iterations and info2.relres < 1e-8
    net.close()
