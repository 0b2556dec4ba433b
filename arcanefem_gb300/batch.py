"""Batched 2D Poisson: host side of ``afem_batch_*``.

A batch is a list of independent Poisson problems on the unit square (the
Poisson module's assemble + eliminate + solve, once per instance), each with
4 right-hand sides made of Gaussian bumps.  The library assembles and solves
all of them in one persistent cooperative launch captured in a CUDA graph;
this module builds the device meshes and structures, owns the outputs, and
runs the autotuner with a JSON cache of its choices.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
import sys

import numpy as np
import torch

from . import _capi, fem, meshgen
from ._capi import call

RHS = 4
BUMPS = 8


class BatchInstance(C.Structure):
    _fields_ = [("nb_node", C.c_int), ("nb_cell", C.c_int), ("coords_d", C.c_void_p), ("cells_d", C.c_void_p),
                ("nc_ptr_d", C.c_void_p), ("nc_cell_d", C.c_void_p), ("nc_local_d", C.c_void_p),
                ("nc_slot_d", C.c_void_p), ("row_ptr_d", C.c_void_p), ("cols_d", C.c_void_p),
                ("dirichlet_d", C.c_void_p), ("sources_d", C.c_void_p), ("values_d", C.c_void_p),
                ("rhs_d", C.c_void_p), ("x_d", C.c_void_p)]


class BatchConfig(C.Structure):
    _fields_ = [("block", C.c_int), ("blocks_per_sm", C.c_int), ("cost_exponent", C.c_float)]

    def as_dict(self):
        return {"block": self.block, "blocks_per_sm": self.blocks_per_sm, "cost_exponent": self.cost_exponent}


class BatchResult(C.Structure):
    _fields_ = [("inner_iterations", C.c_int), ("refinements", C.c_int), ("status", C.c_int),
                ("finish_ms", C.c_float), ("relres", C.c_double * 4)]


def _ptr(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def instance_sizes(count: int = 64, nmin: int = 64, nmax: int = 512, seed: int = 2024) -> list[int]:
    """Square-mesh sides N ~ U{nmin..nmax} (seeded)."""
    rng = np.random.default_rng(seed)
    return [int(v) for v in rng.integers(nmin, nmax + 1, size=count)]


def bump_sources(rng: np.random.Generator) -> np.ndarray:
    """[4][8][4] float32: per right-hand side 8 bumps (amplitude N(0,1),
    centre U[0,1]^2, width U[0.02, 0.1])."""
    s = np.empty((RHS, BUMPS, 4), np.float32)
    s[..., 0] = rng.standard_normal((RHS, BUMPS))
    s[..., 1] = rng.uniform(size=(RHS, BUMPS))
    s[..., 2] = rng.uniform(size=(RHS, BUMPS))
    s[..., 3] = rng.uniform(0.02, 0.1, size=(RHS, BUMPS))
    return s


class Batch:
    """Device meshes, structures and outputs of a batch, and the afem_batch handle."""

    def __init__(self, ctx: fem.Context, sizes: list[int], seed: int = 7, jitter: float = 0.0):
        self.ctx = ctx
        self.sizes = list(sizes)
        rng = np.random.default_rng(seed)
        self.meshes, self.fmts, self.sources, self.dirichlet, self.rhs, self.x = [], [], [], [], [], []
        descs = (BatchInstance * len(sizes))()
        for i, n in enumerate(sizes):
            m = meshgen.unit_square_tri(n, jitter=jitter, seed=seed + i)
            fmt = fem.BSRFormat(ctx, fem.Mesh.from_host(2, m.coords, m.cells))
            fmt.initialize(1)
            fmt.compute_sparsity()
            bnd = np.zeros(m.nb_node, np.uint8)
            bnd[m.groups["boundary"]] = 1
            src = torch.as_tensor(bump_sources(rng), device="cuda").contiguous()
            dbnd = torch.as_tensor(bnd, device="cuda")
            x = torch.zeros((m.nb_node, RHS), dtype=torch.float64, device="cuda")
            b = torch.zeros((m.nb_node, RHS), dtype=torch.float64, device="cuda")
            self.meshes.append(m)
            self.fmts.append(fmt)
            self.sources.append(src)
            self.dirichlet.append(dbnd)
            self.rhs.append(b)
            self.x.append(x)
            fm = fmt.mesh
            descs[i] = BatchInstance(m.nb_node, m.nb_cell, fm.coords.data_ptr(), fm.cells.data_ptr(),
                                     fmt.nc_ptr.data_ptr(), fmt.nc_cell.data_ptr(), fmt.nc_local.data_ptr(),
                                     fmt.nc_slot.data_ptr(), fmt.row_ptr.data_ptr(), fmt.cols.data_ptr(),
                                     dbnd.data_ptr(), src.data_ptr(), fmt.values.data_ptr(), b.data_ptr(),
                                     x.data_ptr())
        h = C.c_void_p()
        call("afem_batch_create", ctx.handle, len(sizes), descs, C.byref(h))
        self.handle = h
        ctx.adopt(self)
        self.nb_node = sum(m.nb_node for m in self.meshes)
        self.nnz = sum(f.nnzb for f in self.fmts)

    def signature(self) -> str:
        return hashlib.sha1(json.dumps(self.sizes).encode()).hexdigest()[:16]

    def config(self):
        cfg = BatchConfig()
        grid = C.c_int()
        call("afem_batch_get_config", self.handle, C.byref(cfg), C.byref(grid))
        return cfg, grid.value

    def set_config(self, block: int, blocks_per_sm: int, cost_exponent: float):
        cfg = BatchConfig(block, blocks_per_sm, cost_exponent)
        call("afem_batch_set_config", self.handle, C.byref(cfg))

    def set_weights(self, weights):
        """Team sizes in proportion to `weights` (None: back to the cost model)."""
        arr = None if weights is None else (C.c_double * len(self.sizes))(*[float(w) for w in weights])
        call("afem_batch_set_weights", self.handle, arr)

    def rebalance(self, options=None, rounds: int = 6, damping: float = 0.5):
        """Feedback partitioning.  Each round estimates every instance's work as
        its measured finish time x its CTAs and moves the weights part of the way
        towards it, w <- w * (work / w)^damping (a full step overshoots: a team's
        speed does not grow in proportion to its CTAs, its barriers cost more);
        all rounds run and the fastest split is kept.  Returns the best launch
        time, its weights (None: the cost model was best) and the finish-time
        spread (min, median, max ms) before and after."""
        opt = options or fem.solver_options(rtol=1e-8, inner_rtol=0.1, max_iter=20000)
        self.set_weights(None)
        res, best_ms = self.solve(opt)
        spread = lambda rr: [float(np.min([r.finish_ms for r in rr])), float(np.median([r.finish_ms for r in rr])),
                             float(np.max([r.finish_ms for r in rr]))]
        before = after = spread(res)
        best_w = None
        w = None
        for _ in range(rounds):
            work = [max(float(res[i].finish_ms), 1e-3) * self.team(i)[1] for i in range(len(self.sizes))]
            w = work if w is None else [wi * (ki / wi) ** damping for wi, ki in zip(w, work)]
            self.set_weights(w)
            res, ms = self.solve(opt)
            if ms < best_ms:
                best_ms, best_w, after = ms, list(w), spread(res)
        self.set_weights(best_w)
        self.last_spread = {"before_ms": before, "after_ms": after}
        return best_ms, best_w

    def team(self, inst: int):
        a, b = C.c_int(), C.c_int()
        call("afem_batch_team", self.handle, inst, C.byref(a), C.byref(b))
        return a.value, b.value

    def solve(self, options: _capi.SolverOptions | None = None):
        res = (BatchResult * len(self.sizes))()
        ms = C.c_float()
        opt = options or fem.solver_options(rtol=1e-8, inner_rtol=0.1, max_iter=20000)
        try:
            call("afem_batch_solve", self.handle, C.byref(opt), res, C.byref(ms))
        except _capi.AfemError as e:   # per-instance statuses and residuals ride on the error
            e.results = list(res)
            raise
        return list(res), float(ms.value)

    def autotune(self, candidates=None, options=None, reps: int = 2, cache: str | None = None, log=None,
                 rebalance: bool = True):
        """Pick the fastest configuration (threads per CTA, CTAs per SM, cost
        exponent) by timing the whole batched launch, then rebalance the teams
        from measured finish times; the choice is cached per (device, batch
        signature) in a JSON file."""
        cache = cache or default_cache_path()
        key = f"{torch.cuda.get_device_name(0)}|{self.signature()}"
        table = {}
        if os.path.exists(cache):
            try:
                with open(cache) as f:
                    table = json.load(f)
            except (OSError, ValueError):
                table = {}
        if key in table:
            c = table[key]
            self.set_config(int(c["block"]), int(c["blocks_per_sm"]), float(c["cost_exponent"]))
            self.set_weights(c.get("weights"))
            return {"cached": True, "config": c, "times_ms": None}
        cands = candidates or default_candidates()
        arr = (BatchConfig * len(cands))(*[BatchConfig(*c) for c in cands])
        times = (C.c_float * len(cands))()
        best = C.c_int()
        opt = options or fem.solver_options(rtol=1e-8, inner_rtol=0.1, max_iter=20000)
        call("afem_batch_autotune", self.handle, C.byref(opt), arr, len(cands), reps, times, C.byref(best))
        chosen = arr[best.value].as_dict()
        if rebalance:
            ms, w = self.rebalance(opt)
            chosen["weights"] = w
            chosen["rebalanced_ms"] = ms
            chosen["team_finish_spread"] = self.last_spread
        table[key] = chosen
        os.makedirs(os.path.dirname(cache) or ".", exist_ok=True)
        tmp = cache + ".tmp"
        with open(tmp, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(tmp, cache)
        if log:
            for c, t in zip(cands, times):
                log(f"  block {c[0]:4d} x {c[1]} per SM, exponent {c[2]:.1f}: {t:9.2f} ms")
        return {"cached": False, "config": chosen, "times_ms": [float(t) for t in times]}

    def failure_test(self, stall_cta: int, spin_limit: int) -> int:
        """Status of a launch in which CTA `stall_cta` never reaches its team barrier."""
        return int(_capi.lib().afem_batch_failure_test(self.handle, stall_cta, C.c_longlong(spin_limit)))

    def close(self):
        if self.handle:
            call("afem_batch_destroy", self.handle)
            self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def default_candidates():
    """(block, CTAs per SM, cost exponent) tried by the autotuner."""
    shapes = [(128, 2), (128, 4), (128, 8), (256, 1), (256, 2), (256, 3), (256, 4), (512, 1), (512, 2)]
    return [(b, k, e) for b, k in shapes for e in (3.0, 3.5)]


def default_cache_path() -> str:
    return os.environ.get("AFEM_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "arcanefem_gb300", "batch_autotune.json"))
