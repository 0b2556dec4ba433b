"""Variable-coefficient diffusion solved with the learned V-cycle preconditioner.

    python -m arcanefem_gb300.examples.learned_fcg [--n 512] [--train] [--solves 2]

-div(k grad u) = f on an n x n triangle grid of the unit square (k = exp of a
Gaussian random field, bump source, u = 0 on the boundary), solved to a 1e-8
FP64 relative residual by flexible CG preconditioned with one V(1,1)-cycle
whose smoothers come from the message-passing network (per-node weights, and
learned factored sparse approximate inverses on the finest and the coarse
levels).  With --train the network is first trained on 2000 solver-generated
pairs (the solver keeps the better parameter set); without it the network
gives its initial smoothers (l1-Jacobi).
"""
from __future__ import annotations

import argparse

import numpy as np
import torch

from arcanefem_gb300 import fem, learned


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--n", type=int, default=512, help="grid cells per side (a power of two)")
    ap.add_argument("--train", action="store_true")
    ap.add_argument("--solves", type=int, default=2)
    ap.add_argument("--seed", type=int, default=7)
    args = ap.parse_args(argv)
    levels = max(3, int(np.log2(args.n)))
    ctx = fem.Context()
    prob, hier, net = learned.setup(ctx, n=args.n, levels=levels, layers=6, seed=args.seed, max_batch=16)
    if args.train:
        R, E = learned.make_training_pairs(prob, count=2000, solves=20, every=25, seed=4)
        rep = learned.train_validated(net, prob, R, E, prob.rhs(np.random.default_rng(77)), epochs=4, batch=16,
                                      lr=2e-3)
        print(f"training: loss {rep['loss'][0]:.4f} -> {rep['loss'][-1]:.4f}, FCG iterations "
              f"{rep['iterations_untrained']} -> {rep['iterations_trained']} (kept {rep['kept']})")
    b = prob.rhs(np.random.default_rng(123))
    for _ in range(args.solves):
        x = torch.zeros_like(b)
        info = net.fcg(prob.row_ptr, prob.cols, prob.values, b, x, fem.solver_options(rtol=1e-8, max_iter=5000))
        print(f"FCG + V-cycle: {info.iterations} iterations, {info.solve_ms:.3f} ms, true relres {info.relres:.2e}")
    net.close()


if __name__ == "__main__":
    main()
