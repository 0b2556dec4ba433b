"""CPU oracle of the learned preconditioner (network, multigrid V-cycle,
loss and gradients).

TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels of afem_mpnn_*.
The reference has no learned preconditioner (it hands the solve to HYPRE /
PETSc / Aleph); this restates the preconditioner the library documents in
include/afem_gb300.h: one symmetric V(1,1)-cycle from a zero initial guess
on the Galerkin hierarchy A_0 = A, A_{l+1} = P_l^T A_l P_l,

    V_l(r):  x1 = d_l * r
             s  = r - A_l x1
             x2 = x1 + P_l V_{l+1}(P_l^T s)
             u  = r - A_l x2
             return x2 + d_l * u           (V_{L-1}(r) = d_{L-1} * r)

with weighted-Jacobi smoothers whose per-node weights come from the network:
    d_l = cap_l * sigmoid(c_l + logit(THETA)),  cap_l = 2 / sum_j |A_l,ij|
    (0 on empty rows), so that 2 diag(d_l)^-1 - A_l is strictly diagonally
    dominant and the V-cycle is symmetric positive definite for any c;
    c = 0 is l1-Jacobi at THETA of the cap;
    c_l = o_l . w_l + beta_l  (o_l the level-l output of the message-passing
    network on the coefficient features x0 = [1, log A_ii - mean log A_ii])

trained on the relative energy norm of the error propagation
||(I - M A) e||_A^2 / ||e||_A^2, with the gradient -2 A (e - M r) of a
symmetric A (as the GPU computes it); the backward pass is the adjoint of
the V-cycle.

Float64 numpy; with ``bf16_round=True`` the values the GPU keeps in BF16
(the 64x64 weights, the activations a, m, o, h and the ReLU-masked
gradients G) are rounded the same way (round to nearest even), so that the
comparison isolates the accumulation order.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

F = 64
THETA = 0.8          # untrained smoother weight, as a fraction of the l1-Jacobi cap


def bf16(x):
    """Round float values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def param_count(NL, L):
    return 3 * F + NL * (2 * F * F + F) + L * (F + 1)


def unpack(params, NL, L):
    p = np.asarray(params, np.float64)
    o = 0
    Win = p[o:o + 2 * F].reshape(2, F); o += 2 * F
    bin_ = p[o:o + F]; o += F
    layers = []
    for _ in range(NL):
        W1 = p[o:o + F * F].reshape(F, F); o += F * F
        W2 = p[o:o + F * F].reshape(F, F); o += F * F
        b = p[o:o + F]; o += F
        layers.append((W1, W2, b))
    heads = []
    for _ in range(L):
        heads.append((p[o:o + F], p[o + F])); o += F + 1
    assert o == p.size, (o, p.size)
    return Win, bin_, layers, heads


def level0_graph(A: sp.csr_matrix):
    d = A.diagonal().copy()
    d[d <= 0] = 1.0
    C = sp.coo_matrix(A)
    w = np.where(C.row == C.col, 0.0, -C.data / np.sqrt(d[C.row] * d[C.col]))
    return sp.csr_matrix((w, (C.row, C.col)), shape=A.shape), d


class Net:
    def __init__(self, A, graphs, restr, prol, layers=None, bf16_round=False):
        self.A = sp.csr_matrix(A)
        self.S0, self.d = level0_graph(A)
        self.S = [self.S0] + list(graphs[1:])
        self.R = restr
        self.P = prol
        self.L = len(self.S)
        self.NL = self.L if layers is None else min(layers, self.L)
        self.q = bf16 if bf16_round else (lambda x: np.asarray(x, np.float64))
        # Galerkin hierarchy A_{l+1} = P_l^T A_l P_l and the smoother base weights
        self.Al = [self.A]
        for l in range(self.L - 1):
            self.Al.append(sp.csr_matrix(self.P[l].T @ self.Al[-1] @ self.P[l]))
        self.base = []          # the caps 2 / ||row||_1
        for Al in self.Al:
            l1 = np.asarray(abs(Al).sum(axis=1)).ravel()
            self.base.append(np.where(l1 > 0, 2.0 / np.where(l1 > 0, l1, 1.0), 0.0))
        logd = np.log(self.d)
        self.x0 = np.stack([np.ones_like(logd), (logd - logd.mean()).astype(np.float32).astype(np.float64)], 1)

    def features(self, params):
        """Network forward: per-level scalings d_l and the activations."""
        q = self.q
        Win, bin_, layers, heads = unpack(params, self.NL, self.L)
        a = q(np.maximum(self.x0 @ Win + bin_, 0))
        c = {"a": a, "h": [a], "m": [], "o": [], "d": []}
        h = a
        for l in range(self.L):
            if l < self.NL:
                W1, W2, b = layers[l]
                m = q(self.S[l] @ h)
                o = q(np.maximum(h @ q(W1) + m @ q(W2) + b, 0))
                c["m"].append(m)
            else:
                o = h
            c["o"].append(o)
            w, beta = heads[l]
            z = np.clip(o @ w + beta + np.log(THETA / (1 - THETA)), -30, 30)
            c["d"].append(self.base[l] / (1 + np.exp(-z)))
            if l + 1 < self.L:
                h = q(self.R[l] @ o)
                c["h"].append(h)
        return c

    def apply(self, d, r):
        """z = M r (one V(1,1)-cycle) and the per-level states (r_l, u_l) the
        backward pass needs."""
        L = self.L
        st = [None] * L

        def V(l, r):
            if l == L - 1:
                st[l] = (r, None)
                return d[l] * r
            A = self.Al[l]
            x1 = d[l] * r
            s = r - A @ x1
            x2 = x1 + self.P[l] @ V(l + 1, self.P[l].T @ s)
            u = r - A @ x2
            st[l] = (r, u)
            return x2 + d[l] * u

        return V(0, r), st

    def adjoint(self, d, st, g):
        """dL/dd_l for dL/dz = g through the V-cycle with states st."""
        L = self.L
        dd = [np.zeros_like(x) for x in d]

        def B(l, g):
            r, u = st[l]
            if l == L - 1:
                dd[l] += g * r
                return d[l] * g
            A = self.Al[l]
            dd[l] += g * u                       # post-smoothing weight
            x2b = g - A @ (d[l] * g)
            sb = self.P[l] @ B(l + 1, self.P[l].T @ x2b)
            x1b = x2b - A @ sb
            dd[l] += x1b * r                     # pre-smoothing weight
            return d[l] * g + sb + d[l] * x1b

        B(0, g)
        return dd

    def forward(self, params, r):
        c = self.features(params)
        return self.apply(c["d"], r)[0]

    def loss_and_grad(self, params, rs, es):
        """Mean relative energy norm of the error propagation,
        ||e - M r||_A^2 / ||e||_A^2 over the (r = A e, e) pairs, and its gradient."""
        c = self.features(params)
        B = len(rs)
        loss = 0.0
        ts, seeds = [], []
        for r, e in zip(rs, es):
            z, t = self.apply(c["d"], r)
            ee = np.dot(e, self.A @ e) + 1e-300
            Av = self.A @ (e - z)
            loss += np.dot(e - z, Av) / ee / B
            ts.append(t)
            seeds.append(-2 * Av / (ee * B))
        return loss, self.backward(params, c, ts, seeds)

    def backward(self, params, c, ts, seeds):
        """Parameter gradient from dL/dz_b (seeds) for z_b = M r_b with V-cycle states ts."""
        q = self.q
        Win, bin_, layers, heads = unpack(params, self.NL, self.L)
        L = self.L
        dd = [np.zeros_like(x) for x in c["d"]]
        for t, s in zip(ts, seeds):
            for l, x in enumerate(self.adjoint(c["d"], t, s)):
                dd[l] += x
        gheads = []
        dO = [None] * L
        for l in range(L):
            dl, cap = c["d"][l], self.base[l]
            dc = dd[l] * dl * (1 - np.where(cap > 0, dl / np.where(cap > 0, cap, 1.0), 0.0))
            w, _ = heads[l]
            gheads.append((c["o"][l].T @ dc, dc.sum()))
            dO[l] = np.outer(dc, w)
        gl = [None] * self.NL
        dh0 = None
        for l in range(L - 1, -1, -1):
            if l >= self.NL:
                dO[l - 1] = dO[l - 1] + self.R[l - 1].T @ dO[l]
                continue
            W1, W2, _ = layers[l]
            G = q(dO[l] * (c["o"][l] > 0))
            gl[l] = (c["h"][l].T @ G, c["m"][l].T @ G, G.sum(0))
            dh = G @ q(W1).T + self.S[l].T @ (G @ q(W2).T)
            if l > 0:
                dO[l - 1] = dO[l - 1] + self.R[l - 1].T @ dh
            else:
                dh0 = dh
        Gin = dh0 * (c["a"] > 0)
        parts = [(self.x0.T @ Gin).ravel(), Gin.sum(0)]
        for g1, g2, gb in gl:
            parts += [g1.ravel(), g2.ravel(), gb]
        for gw, gb in gheads:
            parts += [gw, [gb]]
        return np.concatenate(parts)
