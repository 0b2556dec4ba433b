#!/usr/bin/env python
"""Benchmark: node-wise P1 CSR assembly on one GB300 (assembled nnz/s).

Workload (default): 3D Poisson P1 on the unit cube, 128^3 hexahedra split in
6 tetrahedra (12,582,912 tets, 2,146,689 nodes, 31,802,497 nonzeros),
interior nodes jittered by +-0.15 h (seeded), synthetic data.  A step is one
full assembly of the matrix values (element matrices + node-wise gather) with
the sparsity reused, the AF-BSR / node-wise CSR hot loop of the reference.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One JSON line on rank 0.  ``value`` is device-timed (CUDA events, L2 flushed
between steps); ``e2e`` is the same metric through the public API with host
buffers (mesh in from pinned host memory, connectivity + sparsity + assembly,
CSR back to pinned host memory) inside the timed region.  ``--impl
reference`` times the CPU restatement of the reference's node-wise assembly
(oracle/) on all host cores.  N > 1 runs independent replicas (one per GPU).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "assembled nnz/s (node-wise CSR, 3D Poisson P1)"
UNIT = "nnz/s"
HBM_FALLBACK_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--n", type=int, default=128, help="hexahedra per cube edge")
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    return rank, world, local


def config(args, world):
    return {"workload": f"poisson3d_p1_tet_{args.n}^3 (unit cube, 6-tet Kuhn split, jitter 0.15h)",
            "elements": 6 * args.n ** 3, "nodes": (args.n + 1) ** 3, "seed": args.seed,
            "step": "values assembly (element matrices + node-wise gather), sparsity reused",
            "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{world}",
            "dirichlet": "none in the timed step (matrix only)"}


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def read_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


def read_traffic(name: str):
    """Per-launch DRAM bytes from the committed ncu summary (profiles/), or None."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            m = re.match(r"\s*traffic_bytes_per_assembly\s*[:=]\s*([0-9.eE+]+)", line)
            if m:
                return float(m.group(1))
    except OSError:
        pass
    return None


def algorithmic_bytes(nb_node, nb_cell, nnz, npc=4, dim=3):
    """Values-only assembly bytes: values + coords + cell->node + node->cell (ptr + list)."""
    return 8 * nnz + 8 * dim * nb_node + 4 * npc * nb_cell + 4 * npc * nb_cell + 4 * (nb_node + 1)


# ---------------------------------------------------------------------------
def run_gpu(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    from arcanefem_gb300 import fem, meshgen

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    mesh = meshgen.unit_cube_tet(args.n, jitter=0.15, seed=args.seed)
    ctx = fem.Context()
    dm = fem.Mesh.from_host(3, mesh.coords, mesh.cells)
    fmt = fem.BSRFormat(ctx, dm)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fmt.initialize(1)
    fmt.compute_sparsity()
    torch.cuda.synchronize()
    structure_ms = (time.perf_counter() - t0) * 1e3
    nnz = fmt.nnzb
    ke = torch.empty(fmt.element_planes() * mesh.nb_cell, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step(ev=None):
        if ev:
            ev[0].record()
        fmt.element_matrices(ke)
        if ev:
            ev[1].record()
        fmt.gather(ke)
        if ev:
            ev[2].record()

    for _ in range(max(args.warmup, 3)):
        flush.fill_(1.0)
        step()
    torch.cuda.synchronize()
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    launches0 = ctx.launches
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(float(k))
            step(events[k])
        torch.cuda.synchronize()
        wall_s = time.perf_counter() - t0
    launches = ctx.launches - launches0
    elem_ms = [e[0].elapsed_time(e[1]) for e in events]
    gath_ms = [e[1].elapsed_time(e[2]) for e in events]
    asm_ms = [a + b for a, b in zip(elem_ms, gath_ms)]
    total_ms = sum(asm_ms)
    if world > 1:
        t = torch.tensor([total_ms], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = world * nnz / (ms_per_step * 1e-3)

    # roofline of the assembly (element + gather kernels of one step)
    hbm_peak, peak_kind = read_peaks()
    alg = algorithmic_bytes(mesh.nb_node, mesh.nb_cell, nnz)
    achieved = alg / (ms_per_step * 1e-3) / 1e9
    traffic = read_traffic(f"assembly_poisson_tet_n{args.n}.md")
    fma_rate = ctx.fp64_fma_rate()
    dp_per_tet = 74 + 16      # element kernel + gather adds
    dp_achieved = dp_per_tet * mesh.nb_cell / (ms_per_step * 1e-3) / 1e9

    # e2e: public API, host buffers, transfers inside the timed region
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(args, mesh, nnz)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(mesh, fmt)

    # a cheap correctness guard on the benchmarked output (row sums of a P1 Laplacian vanish)
    vals = fmt.values
    rows = torch.repeat_interleave(torch.arange(mesh.nb_node, device="cuda"), torch.diff(fmt.row_ptr.long()))
    rs = torch.zeros(mesh.nb_node, dtype=torch.float64, device="cuda").index_add_(0, rows, vals)
    row_sum_rel = float(rs.abs().max() / vals.abs().max())

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered mesh)",
            "config": config(args, world),
            "nnz": nnz, "element_ms": statistics.mean(elem_ms), "gather_ms": statistics.mean(gath_ms),
            "structure_ms_once": structure_ms, "wall_s_timed_loop": wall_s, "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved / hbm_peak, "traffic": traffic, "peak_source": peak_kind,
                         "algorithmic_bytes": alg, "kernel": "k_elem_poisson_tet + k_gather_scalar<4>"},
            "fp64_roofline": {"achieved_gdp_instr_s": dp_achieved, "peak_gfma_s": fma_rate,
                              "frac": dp_achieved / fma_rate, "dp_instr_per_tet": dp_per_tet},
            "e2e": e2e, "cpu_baseline": cpu, "clocks": clk.summary(), "check": {"row_sum_rel": row_sum_rel},
        }
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_e2e(args, mesh, nnz):
    import torch

    from arcanefem_gb300 import fem

    coords_h = torch.from_numpy(mesh.coords).pin_memory()
    cells_h = torch.from_numpy(mesh.cells).pin_memory()
    vals_h = torch.empty(nnz, dtype=torch.float64).pin_memory()
    cols_h = torch.empty(nnz, dtype=torch.int32).pin_memory()
    rp_h = torch.empty(mesh.nb_node + 1, dtype=torch.int32).pin_memory()
    ctx = fem.Context()
    dco = torch.empty_like(coords_h, device="cuda")
    dce = torch.empty_like(cells_h, device="cuda")
    ke = torch.empty(10 * mesh.nb_cell, dtype=torch.float64, device="cuda")

    def one():
        dco.copy_(coords_h, non_blocking=True)
        dce.copy_(cells_h, non_blocking=True)
        f = fem.BSRFormat(ctx, fem.Mesh(3, dco, dce))
        f.initialize(1)
        f.compute_sparsity()
        f.element_matrices(ke)
        f.gather(ke)
        rp_h.copy_(f.row_ptr, non_blocking=True)
        cols_h.copy_(f.cols, non_blocking=True)
        vals_h.copy_(f.values, non_blocking=True)
        torch.cuda.current_stream().synchronize()

    steps = max(3, args.steps // 2)
    for _ in range(2):
        one()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        one()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    h2d = coords_h.numel() * 8 + cells_h.numel() * 4
    d2h = nnz * 12 + (mesh.nb_node + 1) * 4
    return {"value": nnz / dt, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": dt * 1e3, "steps": steps,
            "includes": "H2D mesh, node->cell, sparsity, element matrices, gather, D2H CSR"}


def cpu_baseline(mesh, fmt):
    """The oracle's node-wise assembly (CPU restatement of BSRFormat.h:473-537 with
    _computeElementVectorTetra4Gpu) on all host cores, same mesh and sparsity."""
    import numpy as np

    from oracle import oracle as O

    threads = O.max_threads()
    ptr = fmt.nc_ptr.cpu().numpy()
    nc = fmt.nc_cell.cpu().numpy()
    rp = fmt.row_ptr.cpu().numpy()
    cols = fmt.cols.cpu().numpy()
    nnz = int(rp[-1])
    t0 = time.perf_counter()
    v = O.assemble(O.POISSON_TET4, mesh.coords, mesh.cells, ptr, nc, rp, cols, nb_threads=threads)
    dt = time.perf_counter() - t0
    gpu = fmt.values.cpu().numpy()
    err = float(np.max(np.abs(gpu - v) / np.maximum(np.abs(v), 1e-3 * np.abs(v).max())))
    return {"value": nnz / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"one full values assembly of the same mesh ({mesh.nb_cell} tets), {dt:.2f} s",
            "max_rel_diff_vs_gpu": err}


# ---------------------------------------------------------------------------
def run_reference(args):
    """CPU reference arm: the oracle's restatement of the reference node-wise
    assembly, all host threads, rank 0 only."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from arcanefem_gb300 import meshgen
    from oracle import oracle as O

    mesh = meshgen.unit_cube_tet(args.n, jitter=0.15, seed=args.seed)
    ptr, nc, _ = O.node_cell(mesh.nb_node, mesh.cells)
    rp, cols = O.sparsity(mesh.nb_node, mesh.cells)
    nnz = int(rp[-1])
    threads = O.max_threads()
    for _ in range(args.warmup):
        O.assemble(O.POISSON_TET4, mesh.coords, mesh.cells, ptr, nc, rp, cols, nb_threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.assemble(O.POISSON_TET4, mesh.coords, mesh.cells, ptr, nc, rp, cols, nb_threads=threads)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = nnz / (ms * 1e-3)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered mesh)",
           "config": config(args, 1), "impl": "reference",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"full values assembly of the same mesh per step ({mesh.nb_cell} tets)"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "reference (Arcane/HYPRE) cannot be built here; CPU restatement of its node-wise assembly"}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    a = parse_args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_gpu(a)
