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

On the factored levels (the finest level and every level of at most
FACT_ROWS rows) the smoother is a learned factored sparse approximate
inverse instead of d_l * x:

    G_l = theta_l L_l^T L_l,   L_l = (I + N_l) T_l^1/2,   T_l = diag(d_l),
    N_l,ij = m_ij s_i s_j A_l,ij   (strictly lower pattern of A_l; s = sqrt(d_l)),
    m_ij = 2 tanh(o_i . (ew_l * o_j) + eb_l)   (an edge head on the level output),
    theta_l = 1.9 / max(1.9, max_i sum_j |(L_l^T L_l A_l)_ij|),

SPD by construction (L_l lower triangular with a positive diagonal) and with
lambda_max(G_l A_l) < 2 by the row-sum bound, so the V-cycle stays SPD for any
network output; with ew = eb = 0 it is the weighted Jacobi smoother above.
theta_l takes part in the gradient through the row that attains the maximum.

With an exact level (the first level below the finest of at most EXACT_ROWS
rows), the V-cycle stops there and solves it with the inverse of the block of
its nonzero rows (V_ex(r) = A_ex^+ r); the levels below are not used.

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
FACT_ROWS = 2048     # levels of at most this many rows (and the finest) get the factored smoother
EXACT_ROWS = 320     # the first level (below the finest) of at most this many rows is solved exactly
SAFE = 1.9           # the row-sum bound of theta_l G_l A_l


def bf16(x):
    """Round float values to bfloat16 (nearest even), returned as float64."""
    a = np.asarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def exact_level(sizes, exact_rows=EXACT_ROWS):
    """The level solved exactly (the V-cycle stops there), or None: the first
    level below the finest of at most exact_rows rows."""
    if exact_rows is None:
        return None
    for l, n in enumerate(sizes):
        if l > 0 and n <= exact_rows:
            return l
    return None


def fact_levels(sizes, fact_rows=FACT_ROWS, exact=None):
    """The levels that get the factored smoother: the finest and every level of
    at most fact_rows rows (none when fact_rows is None: diagonal smoothers only)."""
    if fact_rows is None:
        return []
    top = len(sizes) if exact is None else exact
    return [l for l, n in enumerate(sizes[:top]) if l == 0 or n <= fact_rows]


def param_count(NL, L, nfact=0):
    return 3 * F + NL * (2 * F * F + F) + L * (F + 1) + nfact * (F + 1)


def unpack(params, NL, L, nfact=0):
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
    edges = []
    for _ in range(nfact):
        edges.append((p[o:o + F], p[o + F])); o += F + 1
    assert o == p.size, (o, p.size)
    return Win, bin_, layers, heads, edges


def level0_graph(A: sp.csr_matrix):
    d = A.diagonal().copy()
    d[d <= 0] = 1.0
    C = sp.coo_matrix(A)
    w = np.where(C.row == C.col, 0.0, -C.data / np.sqrt(d[C.row] * d[C.col]))
    return sp.csr_matrix((w, (C.row, C.col)), shape=A.shape), d


class Net:
    def __init__(self, A, graphs, restr, prol, layers=None, bf16_round=False, fact_rows=None, exact_rows=None):
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
        # exact level: the V-cycle uses levels 0 .. ex and solves level ex with the
        # inverse of its nonzero rows' block (the rows of coarse Dirichlet nodes are empty)
        sizes = [Al.shape[0] for Al in self.Al]
        self.ex = exact_level(sizes, exact_rows)
        self.Lv = self.L if self.ex is None else self.ex + 1
        self.minv = None
        if self.ex is not None:
            Ae = self.Al[self.ex].toarray()
            act = np.abs(Ae).sum(axis=1) > 0
            self.minv = np.zeros_like(Ae)
            self.minv[np.ix_(act, act)] = np.linalg.inv(Ae[np.ix_(act, act)])
        # factored levels: the strictly lower pattern of A_l (row i, column j < i, value A_ij)
        self.fact = fact_levels(sizes, fact_rows, self.ex)
        self.low = {}
        for l in self.fact:
            lo = sp.tril(self.Al[l], k=-1).tocoo()
            keep = lo.data != 0
            self.low[l] = (lo.row[keep], lo.col[keep], lo.data[keep])

    @property
    def nfact(self):
        return len(self.fact)

    def factor(self, l, d, o, ew, eb):
        """The factored smoother of level l: L_l, theta_l and what the backward needs."""
        i, j, a = self.low[l]
        n = self.Al[l].shape[0]
        z = np.einsum("ef,ef,f->e", o[i], o[j], ew) + eb if i.size else np.zeros(0)
        m = 2 * np.tanh(z)
        s = np.sqrt(d[l])
        lval = m * s[i] * s[j] * s[j] * a                       # L_ij = N_ij s_j
        ar = np.arange(n)
        Lf = sp.csr_matrix((np.concatenate([s, lval]), (np.concatenate([ar, i]), np.concatenate([ar, j]))),
                           shape=(n, n))
        LA = sp.csr_matrix(Lf @ self.Al[l])
        GA = sp.csr_matrix(Lf.T @ LA)
        rows = np.asarray(abs(GA).sum(axis=1)).ravel()
        istar = int(np.argmax(rows))
        bound = float(rows[istar])
        theta = SAFE / max(SAFE, bound)
        return {"z": z, "m": m, "s": s, "Lf": Lf, "LA": LA, "GA": GA, "istar": istar, "bound": bound,
                "theta": theta}

    def features(self, params):
        """Network forward: per-level weights d_l, the factored smoothers, and the activations."""
        q = self.q
        Win, bin_, layers, heads, edges = unpack(params, self.NL, self.L, self.nfact)
        a = q(np.maximum(self.x0 @ Win + bin_, 0))
        c = {"a": a, "h": [a], "m": [], "o": [], "d": [], "f": {}}
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
            if l in self.low:
                ew, eb = edges[self.fact.index(l)]
                c["f"][l] = self.factor(l, c["d"], o, ew, eb)
            if l + 1 < self.L:
                h = q(self.R[l] @ o)
                c["h"].append(h)
        return c

    def smooth(self, c, l, x):
        """The level-l smoother applied to x: d_l * x, or theta_l L_l^T L_l x."""
        f = c["f"].get(l)
        if f is None:
            return c["d"][l] * x
        return f["theta"] * (f["Lf"].T @ (f["Lf"] @ x))

    def apply(self, c, r):
        """z = M r (one V(1,1)-cycle) and the per-level states (r_l, u_l) the
        backward pass needs."""
        L = self.Lv
        st = [None] * L

        def V(l, r):
            if l == self.ex:
                st[l] = (r, None)
                return self.minv @ r
            if l == L - 1:
                st[l] = (r, None)
                return self.smooth(c, l, r)
            A = self.Al[l]
            x1 = self.smooth(c, l, r)
            s = r - A @ x1
            x2 = x1 + self.P[l] @ V(l + 1, self.P[l].T @ s)
            u = r - A @ x2
            st[l] = (r, u)
            return x2 + self.smooth(c, l, u)

        return V(0, r), st

    def adjoint(self, c, st, g, acc):
        """Accumulates into acc the gradient of <g, M r> with respect to the
        smoothers: acc["dd"][l] (diagonal levels: dL/dd_l) and, on factored
        levels, acc["gL"][l] (dL/dL_l on its diagonal and lower pattern, as a
        matrix) and acc["dth"][l] (dL/dtheta_l)."""
        L = self.Lv

        def use(l, a, gbar):
            f = c["f"].get(l)
            if f is None:
                acc["dd"][l] += gbar * a
                return
            wa, wg = f["Lf"] @ a, f["Lf"] @ gbar
            acc["dth"][l] += wg @ wa
            # dL/dL_ij = theta (wg_i a_j + wa_i gbar_j) on the pattern of L
            Lf = sp.coo_matrix(f["Lf"])
            acc["gL"][l] += f["theta"] * (wg[Lf.row] * a[Lf.col] + wa[Lf.row] * gbar[Lf.col])

        def B(l, g):
            r, u = st[l]
            if l == self.ex:
                return self.minv @ g                  # no parameter on the exact level
            if l == L - 1:
                use(l, r, g)
                return self.smooth(c, l, g)
            A = self.Al[l]
            use(l, u, g)                              # post-smoothing
            x2b = g - A @ self.smooth(c, l, g)
            sb = self.P[l] @ B(l + 1, self.P[l].T @ x2b)
            x1b = x2b - A @ sb
            use(l, r, x1b)                            # pre-smoothing
            return self.smooth(c, l, g + x1b) + sb

        B(0, g)

    def forward(self, params, r):
        c = self.features(params)
        return self.apply(c, r)[0]

    def loss_and_grad(self, params, rs, es):
        """Mean relative energy norm of the error propagation,
        ||e - M r||_A^2 / ||e||_A^2 over the (r = A e, e) pairs, and its gradient."""
        c = self.features(params)
        B = len(rs)
        loss = 0.0
        ts, seeds = [], []
        for r, e in zip(rs, es):
            z, t = self.apply(c, r)
            ee = np.dot(e, self.A @ e) + 1e-300
            Av = self.A @ (e - z)
            loss += np.dot(e - z, Av) / ee / B
            ts.append(t)
            seeds.append(-2 * Av / (ee * B))
        return loss, self.backward(params, c, ts, seeds)

    def factor_backward(self, l, c, gL, dth, ew):
        """From dL/dL_l (coo order of L_l) and dL/dtheta_l to dL/dd_l, the edge
        head's parameter gradient and its contribution to dL/do_l."""
        f = c["f"][l]
        i, j, a = self.low[l]
        o = c["o"][l]
        Lf = sp.coo_matrix(f["Lf"])
        G = sp.csr_matrix((gL, (Lf.row, Lf.col)), shape=Lf.shape)   # duplicates summed: none on a pattern
        if f["bound"] > SAFE:
            # theta = SAFE / bound: through the row i* that attains the bound
            db = dth * (-SAFE / f["bound"] ** 2)
            ist = f["istar"]
            sign = np.sign(f["GA"].getrow(ist).toarray().ravel())
            Lcsc = sp.csc_matrix(f["Lf"])
            col = Lcsc.getcol(ist).tocoo()                  # entries L_{k i*}
            dG = sp.lil_matrix(Lf.shape)
            LAs = f["LA"] @ sign                            # (L A sign)_k
            As = self.Al[l] @ sign                          # (A sign)_m
            Lcsr = sp.csr_matrix(f["Lf"])
            for k, lk in zip(col.row, col.data):
                dG[k, ist] += LAs[k]
                row = Lcsr.getrow(k).tocoo()
                for mcol in row.col:
                    dG[k, mcol] += lk * As[mcol]
            G = G + db * sp.csr_matrix(dG)
        gd = np.asarray(G.diagonal()).ravel()                # dL/dL_ii = dL/ds_i
        gl = np.asarray(G[i, j]).ravel() if i.size else np.zeros(0)
        s, m = f["s"], f["m"]
        ds = gd.copy()
        # L_ij = m_ij a_ij s_i s_j^2
        if i.size:
            dm = gl * a * s[i] * s[j] ** 2
            np.add.at(ds, i, gl * m * a * s[j] ** 2)
            np.add.at(ds, j, gl * m * a * s[i] * 2 * s[j])
            dz = dm * 2 * (1 - np.tanh(f["z"]) ** 2)
            oij = o[i] * o[j]
            gew = oij.T @ dz
            geb = dz.sum()
            dO = np.zeros_like(o)
            np.add.at(dO, i, dz[:, None] * (ew * o[j]))
            np.add.at(dO, j, dz[:, None] * (ew * o[i]))
        else:
            gew, geb, dO = np.zeros(F), 0.0, np.zeros_like(o)
        dd = np.where(s > 0, ds / (2 * np.where(s > 0, s, 1.0)), 0.0)
        return dd, (gew, geb), dO

    def backward(self, params, c, ts, seeds):
        """Parameter gradient from dL/dz_b (seeds) for z_b = M r_b with V-cycle states ts."""
        q = self.q
        Win, bin_, layers, heads, edges = unpack(params, self.NL, self.L, self.nfact)
        L = self.L
        acc = {"dd": [np.zeros_like(x) for x in c["d"]],
               "gL": {l: np.zeros(c["f"][l]["Lf"].nnz) for l in self.fact}, "dth": {l: 0.0 for l in self.fact}}
        for t, s in zip(ts, seeds):
            self.adjoint(c, t, s, acc)
        dd = acc["dd"]
        gedges = [None] * self.nfact
        dOe = {}
        for k, l in enumerate(self.fact):
            ew, _ = edges[k]
            ddl, gedges[k], dOe[l] = self.factor_backward(l, c, acc["gL"][l], acc["dth"][l], ew)
            dd[l] = dd[l] + ddl
        gheads = []
        dO = [None] * L
        for l in range(L):
            dl, cap = c["d"][l], self.base[l]
            dc = dd[l] * dl * (1 - np.where(cap > 0, dl / np.where(cap > 0, cap, 1.0), 0.0))
            w, _ = heads[l]
            gheads.append((c["o"][l].T @ dc, dc.sum()))
            dO[l] = np.outer(dc, w) + dOe.get(l, 0.0)
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
        for gw, gb in gedges:
            parts += [gw, [gb]]
        return np.concatenate(parts)
