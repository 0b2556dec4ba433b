"""Learned preconditioner: host side of the multilevel message-passing network.

The network, its training kernels and the flexible CG that applies it live in
libafem_gb300.so (``afem_mpnn_*``, ``afem_fcg_solve``).  This module builds
what they need on a structured triangle mesh of the unit square
(``meshgen.unit_square_tri``, node id = i + j (n+1)):

* the level hierarchy: vertex grids of (n/2^l + 1)^2 nodes, 8-neighbour
  graphs (weights 1/8) on the coarse levels for the network, full-weighting
  restriction of its features, the multigrid's bilinear prolongation
  vanishing on the Dirichlet boundary (the grid boundary), and the sparsity
  pattern of each Galerkin coarse operator P^T A P, all as CSR;
* the variable-coefficient diffusion problem -div(k grad u) = f of the
  learned-preconditioner benchmark: k = exp(g), g a Gaussian random field
  (correlation length 0.05, variance 1, FFT on a 1024^2 periodic grid,
  bilinearly sampled at the cell centroids), f a sum of Gaussian bumps,
  u = 0 on the boundary;
* training pairs (r, e) generated by the FEM solver itself: the errors
  e_k = x* - x_k of restarted solver iterates and their residuals A e_k.
"""
from __future__ import annotations

import ctypes as C
import sys

import numpy as np
import scipy.sparse as sp
import torch

from . import _capi, fem, meshgen
from ._capi import call

F = 64


def prolongation(R: sp.csr_matrix) -> sp.csr_matrix:
    """Bilinear interpolation: 4 R^T for full weighting (weight 1 at the
    coinciding node, 1/2 and 1/4 at the edge and cell midpoints)."""
    return sp.csr_matrix(4.0 * R.T)


def _ptr(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def tc_row_gemm(ctx: fem.Context, X1, W1t, X2=None, W2t=None, bias=None, relu=False, out_bf16=True,
                out_f32=False, Yf=None, accumulate=False):
    """The network's layer GEMM on the tcgen05 tensor cores: act(X1 W1 + X2 W2
    + bias) for BF16 X [M, 64] and transposed weights Wt [64, 64] (BF16); returns
    (Yb BF16 or None, Yf FP32 or None)."""
    M = X1.shape[0]
    Yb = torch.empty((M, 64), dtype=torch.bfloat16, device=X1.device) if out_bf16 else None
    if out_f32 and Yf is None:
        Yf = torch.zeros((M, 64), dtype=torch.float32, device=X1.device)
    call("afem_tc_row_gemm", ctx.handle, int(M), _ptr(X1), _ptr(W1t), _ptr(X2), _ptr(W2t), _ptr(bias), int(relu),
         _ptr(Yb), _ptr(Yf), int(accumulate))
    return Yb, Yf


def tc_weight_grad(ctx: fem.Context, X1, X2, G):
    """[X1^T G ; X2^T G] (FP32 [2, 64, 64]) for BF16 [M, 64] inputs, on the tensor cores."""
    dW = torch.empty((2, 64, 64), dtype=torch.float32, device=X1.device)
    call("afem_tc_weight_grad", ctx.handle, int(X1.shape[0]), _ptr(X1), _ptr(X2), _ptr(G), _ptr(dW))
    return dW


# ---------------------------------------------------------------------------
# Structured hierarchy

def grid_graph(m: int) -> sp.csr_matrix:
    """8-neighbour graph of an m x m vertex grid, weight 1/8, symmetric."""
    idx = np.arange(m * m).reshape(m, m)
    rows, cols = [], []
    for dj in (-1, 0, 1):
        for di in (-1, 0, 1):
            if di == 0 and dj == 0:
                continue
            a = idx[max(0, -dj):m - max(0, dj), max(0, -di):m - max(0, di)]
            b = idx[max(0, dj):m - max(0, -dj), max(0, di):m - max(0, -di)]
            rows.append(a.ravel())
            cols.append(b.ravel())
    r = np.concatenate(rows)
    c = np.concatenate(cols)
    return sp.csr_matrix((np.full(r.size, 1.0 / 8.0), (r, c)), shape=(m * m, m * m))


def restriction(mf: int) -> sp.csr_matrix:
    """Full weighting from an mf x mf vertex grid to ((mf-1)/2 + 1)^2."""
    mc = (mf - 1) // 2 + 1
    w1 = {-1: 0.25, 0: 0.5, 1: 0.25}
    rows, cols, vals = [], [], []
    J, I = np.meshgrid(np.arange(mc), np.arange(mc), indexing="ij")
    for dj in (-1, 0, 1):
        for di in (-1, 0, 1):
            fi, fj = 2 * I + di, 2 * J + dj
            ok = (fi >= 0) & (fi < mf) & (fj >= 0) & (fj < mf)
            rows.append((I + J * mc)[ok])
            cols.append((fi + fj * mf)[ok])
            vals.append(np.full(int(ok.sum()), w1[di] * w1[dj]))
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(mc * mc, mf * mf))


def interior_mask(m: int) -> np.ndarray:
    """1 on the interior nodes of an m x m vertex grid, 0 on its boundary."""
    b = np.ones((m, m))
    b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = 0
    return b.ravel()


def masked_prolongation(R: sp.csr_matrix, mf: int) -> sp.csr_matrix:
    """Bilinear prolongation with the rows of fine and the columns of coarse
    boundary nodes removed: the coarse functions satisfy u = 0 there."""
    mc = (mf - 1) // 2 + 1
    return sp.csr_matrix(sp.diags(interior_mask(mf)) @ prolongation(R) @ sp.diags(interior_mask(mc)))


class Hierarchy:
    """Device CSR matrices of the level hierarchy (level 0 = the matrix graph),
    and the sparsity pattern of each Galerkin coarse operator (structure
    only: the values are computed on the device from the matrix)."""

    def __init__(self, n: int, levels: int, row_ptr0: torch.Tensor, cols0: torch.Tensor, dirichlet: bool = True):
        assert n % (1 << (levels - 1)) == 0, "grid size must be divisible by 2^(levels-1)"
        self.levels = levels
        self.sizes = [(n >> l) + 1 for l in range(levels)]
        self.rows = [m * m for m in self.sizes]
        self.keep = []
        dev = "cuda"

        def dcsr(M):
            M = sp.csr_matrix(M)
            M.sort_indices()
            t = (torch.as_tensor(M.indptr.astype(np.int32), device=dev),
                 torch.as_tensor(M.indices.astype(np.int32), device=dev),
                 torch.as_tensor(M.data.astype(np.float32), device=dev))
            self.keep.append(t)
            return t

        self.graph = [(row_ptr0, cols0, None)] + [dcsr(grid_graph(m)) for m in self.sizes[1:]]
        self.restr, self.restrT, self.prol, self.prolT = [], [], [], []
        for l in range(levels - 1):
            R = restriction(self.sizes[l])
            P = masked_prolongation(R, self.sizes[l]) if dirichlet else prolongation(R)
            self.restr.append(dcsr(R))
            self.restrT.append(dcsr(R.T))
            self.prol.append(dcsr(P))
            self.prolT.append(dcsr(P.T))
        rp0, c0 = row_ptr0.cpu().numpy(), cols0.cpu().numpy()
        G = sp.csr_matrix((np.ones(c0.size), c0, rp0), shape=(self.rows[0], self.rows[0]))
        self.coarse = [None]
        for l in range(levels - 1):
            P = sp.csr_matrix(abs(sp.csr_matrix((self.prol[l][2].cpu().numpy(), self.prol[l][1].cpu().numpy(),
                                                 self.prol[l][0].cpu().numpy()),
                                                shape=(self.rows[l], self.rows[l + 1]))))
            G = sp.csr_matrix(P.T @ G @ P)
            G.data[:] = 1.0
            G.sort_indices()
            self.coarse.append(dcsr(G))


class AlgebraicHierarchy:
    """The level hierarchy built from the matrix alone, for any mesh (the
    unstructured triangle and tetrahedron meshes of the reference included):
    smoothed aggregation.

    Per level: strong connections |A_ij| >= theta sqrt(A_ii A_jj); aggregates
    by a greedy pass (a node none of whose strong neighbours is aggregated
    seeds an aggregate with them), then every left-over node joins the
    aggregate of a strong neighbour, or starts its own; the tentative
    prolongation T (1 where a node belongs to an aggregate) is smoothed once,
    P = (I - (4/3) / rho(D^-1 A) D^-1 A) T, with rho estimated by power
    iteration.  Rows with no off-diagonal entry -- the eliminated Dirichlet
    rows, whose matrix row is the identity -- join no aggregate, so P vanishes
    there and the coarse spaces satisfy the boundary condition.  Levels stop
    at `min_coarse` rows.  The network's coarse graphs are the patterns of
    the Galerkin operators with row-normalised weights; its features restrict
    by aggregate averages.  Same attributes as Hierarchy (structure only: the
    library recomputes the coarse values on the device from the matrix).
    Node ids are taken in the matrix's order, so the result is deterministic."""

    def __init__(self, row_ptr0: torch.Tensor, cols0: torch.Tensor, values0: torch.Tensor, levels: int = 12,
                 min_coarse: int = 64, theta: float = 0.08):
        rp = row_ptr0.cpu().numpy()
        c0 = cols0.cpu().numpy()
        v0 = values0.cpu().numpy().astype(np.float64)
        n0 = rp.size - 1
        A = sp.csr_matrix((v0, c0, rp), shape=(n0, n0))
        self.keep = []
        dev = "cuda"

        def dcsr(M):
            M = sp.csr_matrix(M)
            M.sort_indices()
            t = (torch.as_tensor(M.indptr.astype(np.int32), device=dev),
                 torch.as_tensor(M.indices.astype(np.int32), device=dev),
                 torch.as_tensor(M.data.astype(np.float32), device=dev))
            self.keep.append(t)
            return t

        Ps, Ts = [], []
        Al = A
        while Al.shape[0] > min_coarse and len(Ps) + 1 < levels:
            P, T = self._level(Al, theta)
            if P.shape[1] == 0 or P.shape[1] >= Al.shape[0]:
                break
            Ps.append(P)
            Ts.append(T)
            Al = sp.csr_matrix(P.T @ Al @ P)
        self.levels = len(Ps) + 1
        self.rows = [n0] + [P.shape[1] for P in Ps]
        self.sizes = list(self.rows)
        # host copies (scipy) of the transfers and the network's graphs
        self.host_prol, self.host_restr, self.host_graph = list(Ps), [], [None]
        self.graph = [(row_ptr0, cols0, None)]
        self.restr, self.restrT, self.prol, self.prolT = [], [], [], []
        self.coarse = [None]
        G = sp.csr_matrix((np.ones(c0.size), c0, rp), shape=(n0, n0))
        for P, T in zip(Ps, Ts):
            # feature restriction: the average over each aggregate
            cnt = np.asarray(T.sum(axis=0)).ravel()
            R = sp.csr_matrix(sp.diags(1.0 / np.maximum(cnt, 1.0)) @ T.T)
            self.host_restr.append(R)
            self.restr.append(dcsr(R))
            self.restrT.append(dcsr(R.T))
            self.prol.append(dcsr(P))
            self.prolT.append(dcsr(P.T))
            G = sp.csr_matrix(abs(P).T @ G @ abs(P))
            G.data[:] = 1.0
            G.sort_indices()
            self.coarse.append(dcsr(G))
            # the network's graph on this level: the Galerkin pattern without the
            # diagonal, each row averaging its neighbours
            S = sp.csr_matrix(G - sp.diags(G.diagonal()))
            S.eliminate_zeros()
            deg = np.diff(S.indptr)
            S.data = np.repeat(1.0 / np.maximum(deg, 1), deg)
            self.host_graph.append(S)
            self.graph.append(dcsr(S))

    @staticmethod
    def _level(A: sp.csr_matrix, theta: float):
        n = A.shape[0]
        d = A.diagonal()
        C = sp.coo_matrix(A)
        offd = C.row != C.col
        nonzero_offd = np.bincount(C.row[offd & (C.data != 0)], minlength=n)
        dirichlet = nonzero_offd == 0
        strong = offd & (np.abs(C.data) >= theta * np.sqrt(np.abs(d[C.row] * d[C.col])))
        S = sp.csr_matrix((np.ones(int(strong.sum())), (C.row[strong], C.col[strong])), shape=(n, n))
        ind, ptr = S.indices, S.indptr
        agg = np.full(n, -1, np.int64)
        agg[dirichlet] = -2
        na = 0
        for i in range(n):                      # seeds: a node with no aggregated strong neighbour
            if agg[i] != -1:
                continue
            nb = ind[ptr[i]:ptr[i + 1]]
            nb = nb[agg[nb] != -2]
            if np.all(agg[nb] == -1):
                agg[i] = na
                agg[nb] = na
                na += 1
        for i in range(n):                      # left-overs join a strong neighbour's aggregate
            if agg[i] != -1:
                continue
            nb = ind[ptr[i]:ptr[i + 1]]
            cand = agg[nb][agg[nb] >= 0]
            if cand.size:
                agg[i] = cand[0]
        for i in range(n):                      # or start their own
            if agg[i] == -1:
                agg[i] = na
                na += 1
        rows = np.flatnonzero(agg >= 0)
        T = sp.csr_matrix((np.ones(rows.size), (rows, agg[rows])), shape=(n, na))
        dinv = np.where(dirichlet | (d == 0), 0.0, 1.0 / np.where(d != 0, d, 1.0))
        Dinv = sp.diags(dinv)
        x = np.random.default_rng(1).random(n) * (~dirichlet)
        lam = 1.0
        for _ in range(20):                     # rho(D^-1 A) by power iteration
            x = Dinv @ (A @ x)
            lam = float(np.linalg.norm(x))
            if lam == 0.0:
                lam = 1.0
                break
            x /= lam
        P = sp.csr_matrix(T - (4.0 / 3.0 / lam) * (Dinv @ (A @ T)))
        P.eliminate_zeros()
        return P, T


FACT_ROWS = 2048   # the finest level and the levels of at most this many rows get the factored smoother
EXACT_ROWS = 320   # the first level below the finest of at most this many rows is solved exactly


def exact_level(sizes):
    """The level the V-cycle solves exactly (and stops at), or None."""
    for l, n in enumerate(sizes):
        if l > 0 and n <= EXACT_ROWS:
            return l
    return None


def fact_levels(sizes) -> list:
    """The levels whose smoother is the learned factored sparse approximate
    inverse: the finest and those of at most FACT_ROWS rows, above the exact level."""
    ex = exact_level(sizes)
    top = len(sizes) if ex is None else ex
    return [l for l, n in enumerate(sizes[:top]) if l == 0 or n <= FACT_ROWS]


def param_count(layers: int, levels: int, nfact: int = 0) -> int:
    """W_in[2][64], b_in[64]; per layer W1, W2 [64][64], b[64]; per level head
    w[64], beta; per factored level edge head ew[64], eb."""
    return 3 * F + layers * (2 * F * F + F) + levels * (F + 1) + nfact * (F + 1)


def init_params(layers: int, levels: int, seed: int = 0, head_scale: float = 0.01, nfact: int = 0) -> np.ndarray:
    """He-style hidden weights; node heads near zero and edge heads at zero, so
    that the initial preconditioner is the V-cycle with l1-Jacobi smoothing
    (c_l ~ 0, N_l = 0)."""
    rng = np.random.default_rng(seed)
    parts = [rng.normal(0, 1.0, (2, F)), np.zeros(F)]
    for _ in range(layers):
        parts += [rng.normal(0, np.sqrt(1.0 / F), (F, F)), rng.normal(0, np.sqrt(1.0 / F), (F, F)), np.zeros(F)]
    for _ in range(levels):
        parts += [rng.normal(0, head_scale, F), np.zeros(1)]
    for _ in range(nfact):
        parts += [np.zeros(F), np.zeros(1)]
    p = np.concatenate([p.ravel() for p in parts]).astype(np.float32)
    assert p.size == param_count(layers, levels, nfact)
    return p


class MPNN:
    """ctypes wrapper of the afem_mpnn handle."""

    def __init__(self, ctx: fem.Context, hier: Hierarchy, layers: int = 6, max_batch: int = 8):
        self.ctx = ctx
        self.hier = hier
        L = hier.levels
        layers = min(layers, L)
        P = C.c_void_p

        def arr(items, k):
            return (P * L)(*[P(0 if it is None or it[k] is None else it[k].data_ptr()) for it in items] +
                           [P(0)] * (L - len(items)))

        h = P()
        sizes = (C.c_int * L)(*hier.rows)
        args = [arr(hier.graph, 0), arr(hier.graph, 1), arr(hier.graph, 2)]
        for mats in (hier.restr, hier.restrT, hier.prol, hier.prolT):
            args += [arr(mats, 0), arr(mats, 1), arr(mats, 2)]
        args += [arr(hier.coarse, 0), arr(hier.coarse, 1)]
        L_ = _capi.lib()
        L_.afem_mpnn_create.restype = C.c_int
        rc = L_.afem_mpnn_create(ctx.handle, C.c_int(L), C.c_int(layers), sizes, *args, C.c_int(max_batch),
                                 C.byref(h))
        _capi.check(rc, "afem_mpnn_create")
        self.handle = h
        ctx.adopt(self)
        self.max_batch = max_batch
        self.nparam = int(_capi.lib().afem_mpnn_param_count(h))
        self.n0 = hier.rows[0]
        self.levels = L
        self.layers = layers
        # edge heads of the factored levels (the finest and those of at most FACT_ROWS rows)
        self.nfact = (self.nparam - param_count(layers, L)) // (F + 1)
        assert self.nfact == len(fact_levels(hier.rows)), (self.nfact, hier.rows)

    def init_params(self, seed: int = 0, head_scale: float = 0.01, edge_scale: float = 0.0) -> np.ndarray:
        """Initial parameters of this network (init_params); with edge_scale > 0
        the edge heads get N(0, edge_scale) weights and biases instead of zeros."""
        p = init_params(self.layers, self.levels, seed=seed, head_scale=head_scale, nfact=self.nfact)
        if edge_scale > 0:
            k = param_count(self.layers, self.levels)
            p[k:] = np.random.default_rng(seed + 1).normal(0, edge_scale, p.size - k).astype(np.float32)
        return p

    def set_params(self, p):
        t = torch.as_tensor(np.asarray(p, np.float32), device="cuda")
        call("afem_mpnn_set_params", self.handle, _ptr(t))

    def get_params(self) -> np.ndarray:
        t = torch.empty(self.nparam, dtype=torch.float32, device="cuda")
        call("afem_mpnn_get_params", self.handle, _ptr(t))
        return t.cpu().numpy()

    def set_operator(self, row_ptr, cols, values):
        call("afem_mpnn_set_operator", self.handle, int(row_ptr.numel()) - 1, _ptr(row_ptr), _ptr(cols),
             _ptr(values))

    def set_coarse_rows(self, rows: int):
        call("afem_mpnn_set_coarse_rows", self.handle, int(rows))

    def scalings(self, level: int) -> torch.Tensor:
        d = torch.empty(self.hier.rows[level], dtype=torch.float32, device="cuda")
        call("afem_mpnn_scalings", self.handle, level, _ptr(d))
        return d

    def forward(self, r: torch.Tensor) -> torch.Tensor:
        b = r.numel() // self.n0
        z = torch.empty_like(r, dtype=torch.float32)
        call("afem_mpnn_forward", self.handle, b, _ptr(r.contiguous()), _ptr(z))
        return z

    def gradients(self, r, e):
        b = r.numel() // self.n0
        g = torch.empty(self.nparam, dtype=torch.float32, device="cuda")
        loss = C.c_double()
        call("afem_mpnn_gradients", self.handle, b, _ptr(r.contiguous()), _ptr(e.contiguous()), _ptr(g),
             C.byref(loss))
        return g, float(loss.value)

    def train_step(self, r, e, lr):
        b = r.numel() // self.n0
        loss = C.c_double()
        call("afem_mpnn_train_step", self.handle, b, _ptr(r.contiguous()), _ptr(e.contiguous()), C.c_float(lr),
             C.byref(loss))
        return float(loss.value)

    def fcg(self, row_ptr, cols, values, b, x, options=None) -> _capi.SolveInfo:
        info = _capi.SolveInfo()
        opt = options or fem.solver_options()
        return fem.solve_call("afem_fcg_solve", info, self.ctx.handle, int(row_ptr.numel()) - 1, _ptr(row_ptr),
                              _ptr(cols), _ptr(values), _ptr(b), _ptr(x), self.handle, C.byref(opt), C.byref(info))

    def close(self):
        if self.handle:
            call("afem_mpnn_destroy", self.handle)
            self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# The variable-coefficient diffusion problem

def gaussian_random_field(seed: int, corr: float = 0.05, var: float = 1.0, grid: int = 1024) -> np.ndarray:
    """Periodic GRF on [0,1)^2 with Gaussian covariance exp(-d^2 / (2 corr^2)), unit variance."""
    rng = np.random.default_rng(seed)
    k = np.fft.fftfreq(grid, d=1.0 / grid)
    kx, ky = np.meshgrid(k, k, indexing="ij")
    spec = np.exp(-0.5 * (2 * np.pi * corr) ** 2 * (kx ** 2 + ky ** 2))
    noise = rng.standard_normal((grid, grid)) + 1j * rng.standard_normal((grid, grid))
    g = np.real(np.fft.ifft2(np.sqrt(spec) * noise))
    g = (g - g.mean()) / g.std() * np.sqrt(var)
    return g


def sample_bilinear(field: np.ndarray, x: np.ndarray, y: np.ndarray) -> np.ndarray:
    n = field.shape[0]
    fx, fy = (x % 1.0) * n, (y % 1.0) * n
    i0, j0 = np.floor(fx).astype(int) % n, np.floor(fy).astype(int) % n
    i1, j1 = (i0 + 1) % n, (j0 + 1) % n
    tx, ty = fx - np.floor(fx), fy - np.floor(fy)
    return ((1 - tx) * (1 - ty) * field[i0, j0] + tx * (1 - ty) * field[i1, j0] + (1 - tx) * ty * field[i0, j1] +
            tx * ty * field[i1, j1])


def bumps(rng, x, y, count=8):
    """sum of `count` Gaussian bumps: amplitudes N(0,1), centres U[0,1]^2, widths U[0.02, 0.1]."""
    f = np.zeros_like(x)
    for _ in range(count):
        a, cx, cy, w = rng.standard_normal(), rng.uniform(), rng.uniform(), rng.uniform(0.02, 0.1)
        f += a * np.exp(-((x - cx) ** 2 + (y - cy) ** 2) / (2 * w * w))
    return f


class DiffusionProblem:
    """Assembled -div(k grad u) = f on the unit square, u = 0 on the boundary."""

    def __init__(self, ctx: fem.Context, n: int = 512, seed: int = 7, jitter: float = 0.2):
        self.ctx = ctx
        self.n = n
        self.mesh = meshgen.unit_square_tri(n, jitter=jitter, seed=seed)
        m = self.mesh
        cent = m.coords[m.cells].mean(axis=1)
        g = gaussian_random_field(seed + 1)
        self.k = np.exp(sample_bilinear(g, cent[:, 0], cent[:, 1]))
        self.fmt = fem.BSRFormat(ctx, fem.Mesh.from_host(2, m.coords, m.cells))
        self.fmt.initialize(1)
        self.fmt.compute_sparsity()
        self.fmt.assemble_poisson(torch.as_tensor(self.k, device="cuda"))
        self.boundary = torch.as_tensor(m.groups["boundary"], device="cuda")
        ls = fem.DoFLinearSystem(ctx, m.nb_node)
        self.fmt.to_linear_system(ls)
        ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, self.boundary, 1, 0, 0.0)
        ls.apply_matrix_transformation()
        self.ls = ls
        self.row_ptr, self.cols, self.values = self.fmt.to_csr()
        # lumped load weights: sum of area / 3 over the incident cells
        w = torch.zeros(m.nb_node, dtype=torch.float64, device="cuda")
        self.fmt.rhs_constant_source(1.0, w)
        self.lumped = w
        self.interior = torch.ones(m.nb_node, dtype=torch.float64, device="cuda")
        self.interior[self.boundary.long()] = 0.0

    def rhs(self, rng) -> torch.Tensor:
        f = bumps(rng, self.mesh.coords[:, 0], self.mesh.coords[:, 1])
        return self.lumped * torch.as_tensor(f, device="cuda") * self.interior

    def apply(self, x: torch.Tensor) -> torch.Tensor:
        y = torch.empty_like(x)
        fem.spmv_csr(self.ctx, self.row_ptr, self.cols, self.values, x, y)
        return y

    def cg(self, b, rtol=1e-8, max_iter=20000, precision=fem.PRECISION_FP64):
        x = torch.zeros_like(b)
        info = fem.cg_solve_csr(self.ctx, self.row_ptr, self.cols, self.values, b, x,
                                options=fem.solver_options(rtol=rtol, max_iter=max_iter, precision=precision))
        return x, info


def cg_steps(prob: DiffusionProblem, b: torch.Tensor, x: torch.Tensor, iters: int) -> None:
    """`iters` iterations of Jacobi FP64 CG from the current x (a restart)."""
    info = _capi.SolveInfo()
    opt = fem.solver_options(rtol=1e-300, max_iter=iters)
    rc = _capi.lib().afem_cg_solve_csr(prob.ctx.handle, int(prob.row_ptr.numel()) - 1, _ptr(prob.row_ptr),
                                       _ptr(prob.cols), _ptr(prob.values), _ptr(b), _ptr(x), _ptr(None),
                                       C.byref(opt), C.byref(info))
    if rc not in (0, _capi.NOT_CONVERGED):
        _capi.check(rc, "afem_cg_solve_csr")


def fcg_steps(net: MPNN, prob: DiffusionProblem, b: torch.Tensor, x: torch.Tensor, iters: int) -> None:
    """`iters` iterations of flexible CG preconditioned by the network, from
    the current x (a restart)."""
    info = _capi.SolveInfo()
    opt = fem.solver_options(rtol=1e-300, max_iter=iters)
    rc = _capi.lib().afem_fcg_solve(prob.ctx.handle, int(prob.row_ptr.numel()) - 1, _ptr(prob.row_ptr),
                                    _ptr(prob.cols), _ptr(prob.values), _ptr(b), _ptr(x), net.handle,
                                    C.byref(opt), C.byref(info))
    if rc not in (0, _capi.NOT_CONVERGED):
        _capi.check(rc, "afem_fcg_solve")


def make_training_pairs(prob: DiffusionProblem, count: int, solves: int, every: int = 25, seed: int = 11,
                        net: MPNN = None):
    """`count` (residual, error) pairs generated by the solver: for each of
    `solves` bump right-hand sides b, the converged solution x* (to 1e-10)
    and the iterates x_k of a solver restarted every `every` iterations from
    x_0 = 0 -- Jacobi CG, or flexible CG preconditioned by `net` when given;
    the pair is (r_k = A e_k, e_k = x* - x_k), so early pairs carry the
    initial errors and late ones the errors the solver is slow to remove."""
    rng = np.random.default_rng(seed)
    n = prob.mesh.nb_node
    R = torch.empty((count, n), dtype=torch.float32, device="cuda")
    E = torch.empty((count, n), dtype=torch.float32, device="cuda")
    per = -(-count // solves)
    s = 0
    while s < count:
        b = prob.rhs(rng)
        if net is None:
            xs, _ = prob.cg(b, rtol=1e-10)
        else:
            xs = torch.zeros_like(b)
            net.fcg(prob.row_ptr, prob.cols, prob.values, b, xs, fem.solver_options(rtol=1e-10, max_iter=5000))
        x = torch.zeros_like(b)
        for k in range(per):
            if s >= count:
                break
            if k:
                if net is None:
                    cg_steps(prob, b, x, every)
                else:
                    fcg_steps(net, prob, b, x, every)
            e = xs - x
            R[s] = prob.apply(e).float()
            E[s] = e.float()
            s += 1
    return R, E


def train(net: MPNN, R, E, epochs=6, batch=8, lr=2e-3, seed=0, log=None):
    """Adam on the mean relative squared error; returns the per-epoch mean loss."""
    rng = np.random.default_rng(seed)
    count = R.shape[0]
    hist = []
    step = 0
    total = epochs * (count // batch)
    for ep in range(epochs):
        perm = rng.permutation(count)
        losses = []
        for i in range(0, count - batch + 1, batch):
            idx = torch.as_tensor(perm[i:i + batch], device="cuda")
            cur = lr * 0.5 * (1 + np.cos(np.pi * step / max(total, 1)))   # cosine decay
            losses.append(net.train_step(R[idx], E[idx], cur))
            step += 1
        hist.append(float(np.mean(losses)))
        if log:
            log(f"epoch {ep}: loss {hist[-1]:.4f}")
    return hist


def train_validated(net: MPNN, prob: DiffusionProblem, R, E, b_val, epochs=6, batch=16, lr=2e-3, rtol=1e-8,
                    log=None):
    """Train, then let the solver judge: FCG on the held-out right-hand side
    b_val with the parameters before and after training; the ones that reach
    rtol in fewer iterations stay in the network.  Returns the loss history
    and both iteration counts."""
    opt = fem.solver_options(rtol=rtol, max_iter=20000)
    before = net.get_params()
    x = torch.zeros_like(b_val)
    it_before = net.fcg(prob.row_ptr, prob.cols, prob.values, b_val, x, opt).iterations
    hist = train(net, R, E, epochs=epochs, batch=batch, lr=lr, log=log)
    x = torch.zeros_like(b_val)
    it_after = net.fcg(prob.row_ptr, prob.cols, prob.values, b_val, x, opt).iterations
    kept = "trained"
    if it_after > it_before:
        net.set_params(before)
        kept = "untrained"
    return {"loss": hist, "iterations_untrained": it_before, "iterations_trained": it_after, "kept": kept}


def setup(ctx: fem.Context, n=512, levels=9, layers=6, seed=7, max_batch=8):
    prob = DiffusionProblem(ctx, n=n, seed=seed)
    hier = Hierarchy(n, levels, prob.row_ptr, prob.cols)
    net = MPNN(ctx, hier, layers=layers, max_batch=max_batch)
    net.set_params(net.init_params(seed))
    net.set_operator(prob.row_ptr, prob.cols, prob.values)
    return prob, hier, net
