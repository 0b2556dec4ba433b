#!/usr/bin/env python
"""Benchmark: node-wise P1 assembly on one GB300 (assembled nnz/s), plus the
time to a relative residual of the Krylov solve on the assembled system.

Workloads (synthetic, seeded jittered structured meshes):
  poisson3d    (default) 3D Poisson P1, unit cube 128^3 hexahedra x 6 tets
               (12,582,912 tets, 2,146,689 nodes, 31,802,497 nnz); f = 1,
               u = 0 on x = 0 and x = 1; CG to 1e-8.
  elasticity3d linear elasticity P1, 96^3 x 6 tets, 3x3 blocks
               (121,188,969 scalar nnz); E = 21e5, nu = 0.28, f = (0,0,-1),
               clamped at z = 0; mixed-precision CG to 1e-8.
  poisson2d    2D Poisson P1, 256^2 quads x 2 tris; f = -1, u = 0 on the
               boundary; CG to 1e-10.

A step is one full assembly of the matrix values (element matrices +
node-wise gather) with the sparsity reused: the node-wise CSR / AF-BSR hot
loop of the reference.

Two more sections ride on the same line (rank 0):
  learned  512^2 variable-coefficient diffusion: time to 1e-8 of plain FP64
           CG against flexible CG with the learned V-cycle preconditioner;
  batched  64 Poisson instances (N ~ U{64..512}) x 4 right-hand sides,
           assembled and solved to 1e-8 in one persistent launch.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--workload poisson3d|elasticity3d|poisson2d]

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
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

UNIT = "nnz/s"
HBM_FALLBACK_GBS = 6800.0

WORKLOADS = {
    "poisson3d": dict(dim=3, n=128, jitter=0.15, nb_dof=1, metric="assembled nnz/s (node-wise CSR, 3D Poisson P1)",
                      dp_gather=16, rtol=1e-8, precision="fp64", dirichlet="x_faces", source=1.0),
    "elasticity3d": dict(dim=3, n=96, jitter=0.15, nb_dof=3,
                         metric="assembled nnz/s (node-wise 3x3 BSR, 3D linear elasticity P1)",
                         dp_gather=144, rtol=1e-8, precision="mixed", dirichlet="zmin",
                         E=21e5, nu=0.28, body=(0.0, 0.0, -1.0)),
    "poisson2d": dict(dim=2, n=256, jitter=0.2, nb_dof=1, metric="assembled nnz/s (node-wise CSR, 2D Poisson P1)",
                      dp_gather=9, rtol=1e-10, precision="fp64", dirichlet="boundary", source=-1.0),
    # Q1 widening: trilinear hexahedra (2x2x2 Gauss points), Q1 source, FP64 / mixed CG
    "poisson3d_hex": dict(dim=3, cell="hex", n=96, jitter=0.15, nb_dof=1,
                          metric="assembled nnz/s (node-wise CSR, 3D Poisson Q1 Hexa8)",
                          dp_gather=64, rtol=1e-8, precision="fp64", dirichlet="x_faces", source=1.0),
}
# the workloads that ride along on the default line, after the main one
EXTRA_WORKLOADS = ("elasticity3d", "poisson2d", "poisson3d_hex")
FORMULATIONS = ("reference", "minimal")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    p.add_argument("--workload", choices=list(WORKLOADS), default="poisson3d")
    p.add_argument("--n", type=int, default=0, help="elements per edge (default: the workload's)")
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--e2e-chunks", type=int, default=0,
                   help="cell ranges of the e2e assembly / copy-back overlap (0: the library's choice, "
                        "one per ~80 MB of values, at most 12; 1..16)")
    p.add_argument("--no-solve", action="store_true")
    p.add_argument("--inner-rtol", type=float, default=0.1,
                   help="mixed precision: FP32 CG residual reduction between reliable updates")
    p.add_argument("--no-learned", action="store_true", help="skip the learned-preconditioner section")
    p.add_argument("--no-batched", action="store_true", help="skip the batched-solve section")
    p.add_argument("--learned-n", type=int, default=512)
    p.add_argument("--batched-count", type=int, default=64)
    p.add_argument("--batched-sides", type=int, nargs=2, default=(64, 512), metavar=("MIN", "MAX"))
    p.add_argument("--batched-tune", choices=["auto", "none"], default="auto",
                   help="auto: autotune (JSON cache); none: the library's default configuration")
    p.add_argument("--no-extra-workloads", action="store_true",
                   help="measure the main workload only (skip " + ", ".join(EXTRA_WORKLOADS) + ")")
    a = p.parse_args()
    if a.n <= 0:
        a.n = WORKLOADS[a.workload]["n"]
    return a


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def replica_value(total_ms: float, world: int, units_per_rank: int, steps: int, device: str):
    """Replicas: every rank assembled its own copy; the job time is the max
    over ranks and the value is all ranks' units over that time."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([total_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / steps
    return ms_per_step, world * units_per_rank / (ms_per_step * 1e-3)


def make_mesh(name, n, seed):
    from arcanefem_gb300 import meshgen
    w = WORKLOADS[name]
    if w.get("cell") == "hex":
        return meshgen.unit_cube_hex(n, jitter=w["jitter"], seed=seed)
    if w["dim"] == 3:
        return meshgen.unit_cube_tet(n, jitter=w["jitter"], seed=seed)
    return meshgen.unit_square_tri(n, jitter=w["jitter"], seed=seed)


def config(name, n, seed, world):
    w = WORKLOADS[name]
    if w.get("cell") == "hex":
        desc = f"unit cube {n}^3 trilinear hexahedra, jitter {w['jitter']}h"
        elements, nodes = n ** 3, (n + 1) ** 3
    elif w["dim"] == 3:
        desc = f"unit cube {n}^3 hexahedra x 6 Kuhn tetrahedra, jitter {w['jitter']}h"
        elements, nodes = 6 * n ** 3, (n + 1) ** 3
    else:
        desc = f"unit square {n}^2 quads x 2 triangles, jitter {w['jitter']}h"
        elements, nodes = 2 * n ** 2, (n + 1) ** 2
    return {"workload": f"{name} ({desc})", "elements": elements, "nodes": nodes,
            "dof_per_node": w["nb_dof"], "seed": seed,
            "step": "values assembly (element matrices + node-wise gather), sparsity reused",
            "element_arithmetic": "reference rounding (bit-identical to the reference's node-wise assembly)",
            "l2": "flushed between steps (256 MB write)", "parallelism": f"replicas x{world}"}


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
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.2)
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
    try:
        d = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return HBM_FALLBACK_GBS, "fallback"


def read_counters(name: str, n: int, formulation: str):
    """ncu counters of one assembly of this workload (profiles/assembly_counters.json,
    machine-readable; the capture commands are recorded in it): DRAM bytes per
    assembly and FP64 instructions per cell, or {} when not captured."""
    try:
        with open(os.path.join(ROOT, "profiles", "assembly_counters.json")) as f:
            table = json.load(f)
        return dict(table["workloads"][f"{name}_n{n}"][formulation])
    except (OSError, KeyError, ValueError, TypeError):
        return {}


def algorithmic_bytes(mesh, nnz_scalar):
    """Values-only assembly bytes: values + coords + cell->node + node->cell (list + ptr)."""
    npc, n, c = mesh.npc, mesh.nb_node, mesh.nb_cell
    return 8 * nnz_scalar + 8 * 3 * n + 4 * npc * c + 4 * npc * c + 4 * (n + 1)


# ---------------------------------------------------------------------------
def time_assembly(fmt, ke, lam, mu, steps, warmup, flush, clk_index=None):
    """Device time of the values assembly (element matrices, then the node-wise
    gather), CUDA events on the launching stream around each stage, L2 flushed
    before every step; nvidia-smi clocks sampled over the timed region when
    clk_index is given."""
    import contextlib

    import torch

    def step(ev=None):
        if ev:
            ev[0].record()
        fmt.element_matrices(ke, lam=lam, mu=mu)
        if ev:
            ev[1].record()
        fmt.gather(ke)
        if ev:
            ev[2].record()

    for _ in range(max(warmup, 3)):
        flush.fill_(1.0)
        step()
    torch.cuda.synchronize()
    events = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    launches0 = fmt.ctx.launches
    clk = ClockSampler(clk_index) if clk_index is not None else contextlib.nullcontext()
    with clk:
        t0 = time.perf_counter()
        for k in range(steps):
            flush.fill_(float(k))
            step(events[k])
        torch.cuda.synchronize()
        wall_s = time.perf_counter() - t0
    fmt.ctx.synchronize()   # raises on a degenerate cell
    elem = [e[0].elapsed_time(e[1]) for e in events]
    gath = [e[1].elapsed_time(e[2]) for e in events]
    return {"element_ms": elem, "gather_ms": gath, "total_ms": sum(a + b for a, b in zip(elem, gath)),
            "launches": fmt.ctx.launches - launches0, "wall_s": wall_s,
            "clocks": clk.summary() if clk_index is not None else None}


def time_structure(fmt, reps=3):
    """Warm device time (CUDA events) of the structure build on the existing
    buffers: node -> cell lists, row lengths + scan, columns + slot map."""
    import ctypes as C

    import torch

    from arcanefem_gb300._capi import call
    m = fmt.mesh
    p = lambda t: C.c_void_p(t.data_ptr())
    nnz = C.c_int64()
    res = {"node_cell_ms": [], "rows_ms": [], "cols_ms": []}
    for _ in range(reps + 1):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record()
        call("afem_node_cell_build", fmt.ctx.handle, m.nb_node, m.nb_cell, m.npc, p(m.cells), p(fmt.nc_ptr),
             p(fmt.nc_cell), p(fmt.nc_local), p(fmt.nc_inverse))
        ev[1].record()
        call("afem_sparsity_rows", fmt.ctx.handle, m.nb_node, m.npc, p(m.cells), p(fmt.nc_ptr), p(fmt.nc_cell),
             p(fmt.row_ptr), C.byref(nnz))
        ev[2].record()
        call("afem_sparsity_cols", fmt.ctx.handle, m.nb_node, m.npc, p(m.cells), p(fmt.nc_ptr), p(fmt.nc_cell),
             p(fmt.nc_local), p(fmt.row_ptr), fmt.col_order, p(fmt.cols), p(fmt.nc_slot))
        ev[3].record()
        torch.cuda.synchronize()
        for k, key in enumerate(("node_cell_ms", "rows_ms", "cols_ms")):
            res[key].append(ev[k].elapsed_time(ev[k + 1]))
    out = {k: statistics.median(v[1:]) for k, v in res.items()}
    out["sparsity_ms"] = out["rows_ms"] + out["cols_ms"]
    out["note"] = "warm, device time; rows_ms includes the host read of nnz"
    if fmt.nb_dof > 1:   # BSRMatrix::toCsr: the block structure expanded to scalar rows on the device
        times = []
        for _ in range(reps + 1):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
            ev[0].record()
            fmt.to_csr()
            ev[1].record()
            torch.cuda.synchronize()
            times.append(ev[0].elapsed_time(ev[1]))
        out["bsr_to_csr_ms"] = statistics.median(times[1:])
    return out


def kernel_names(name, mesh, formulation):
    w = WORKLOADS[name]
    if w["nb_dof"] == 3:
        return "k_elem_elasticity_tet + k_gather_elasticity"
    if w.get("cell") == "hex":
        return "k_elem_poisson_hexa8 + k_gather_scalar<8>"
    if formulation == "minimal":
        return f"k_elem_poisson_{'tet' if mesh.dim == 3 else 'tri'} + k_gather_scalar<{mesh.npc}>"
    return f"k_elem_poisson_p1_ref<{mesh.npc}> + k_gather_scalar<{mesh.npc}>"


def measure_workload(args, name, n, ctx, rank, world, local, main):
    """One workload: structure once, then the timed values assembly in the
    reference rounding (the headline) and in the minimal-instruction
    formulation, each checked against the oracle; e2e through the public API
    with host buffers; the solves."""
    import torch

    from arcanefem_gb300 import fem

    w = WORKLOADS[name]
    mesh = make_mesh(name, n, args.seed)
    dm = fem.Mesh.from_host(mesh.dim, mesh.coords, mesh.cells)
    fmt = fem.BSRFormat(ctx, dm)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fmt.initialize(w["nb_dof"])
    fmt.compute_sparsity()
    torch.cuda.synchronize()
    structure_ms = (time.perf_counter() - t0) * 1e3
    nnz = fmt.nnzb * w["nb_dof"] ** 2
    lam, mu = fem.lame(w["E"], w["nu"]) if w["nb_dof"] == 3 else (0.0, 0.0)
    ke = torch.empty(fmt.element_buffer_size(), dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    steps = args.steps if main else min(args.steps, 10)

    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    ctx.formulation = fem.FORMULATION_REFERENCE
    t_ref = time_assembly(fmt, ke, lam, mu, steps, args.warmup, flush, clk_index=local)
    ms_per_step, value = replica_value(t_ref["total_ms"], world, nnz, steps, "cuda")

    hbm_peak, peak_kind = read_peaks()
    alg = algorithmic_bytes(mesh, nnz)
    fma_rate = ctx.fp64_fma_rate()

    def rooflines(ms, formulation):
        counters = read_counters(name, n, formulation)
        achieved = alg / (ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                "traffic": counters.get("traffic_bytes_per_assembly"), "peak_source": peak_kind,
                "algorithmic_bytes": alg, "kernel": kernel_names(name, mesh, formulation),
                "limiter": "fp64 issue (fp64_roofline): the element arithmetic is FP64 on a part with a "
                           "narrow FP64 pipe"}
        dp_cell = counters.get("fp64_instructions_per_cell")
        fp = None
        if dp_cell:
            dp_achieved = dp_cell * mesh.nb_cell / (ms * 1e-3) / 1e9
            fp = {"achieved_g_fp64_instr_s": dp_achieved, "peak_g_fma_s": fma_rate, "frac": dp_achieved / fma_rate,
                  "fp64_instructions_per_cell": dp_cell,
                  "source": "ncu thread-level DADD+DFMA+DMUL per cell (profiles/assembly_counters.json); peak: "
                            "afem_device_fp64_fma_rate measured on this GPU in this run"}
            if fp["frac"] > roof["frac"]:
                # the FP64 pipe binds: it is the line's roofline, the HBM figures stay beside it
                hbm = {k: roof[k] for k in ("achieved", "peak", "unit", "frac", "peak_source")}
                roof = {"bound": "fp64", "achieved": dp_achieved, "peak": fma_rate, "unit": "G FP64 instr/s",
                        "frac": fp["frac"], "traffic": roof["traffic"], "peak_source": "measured (FP64 FMA loop)",
                        "algorithmic_bytes": alg, "kernel": roof["kernel"], "hbm": hbm,
                        "fp64_instructions_per_cell": dp_cell}
        return roof, fp

    roof, fp64 = rooflines(ms_per_step, "reference")
    out = {"value": value, "unit": UNIT, "ms_per_step": ms_per_step, "steps": steps, "nnz": nnz,
           "config": config(name, n, args.seed, world),
           "element_ms": statistics.mean(t_ref["element_ms"]), "gather_ms": statistics.mean(t_ref["gather_ms"]),
           "structure_ms_once": structure_ms, "wall_s_timed_loop": t_ref["wall_s"],
           "gpu_launches": t_ref["launches"], "roofline": roof, "fp64_roofline": fp64, "clocks": t_ref["clocks"]}

    oracle_values = None
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"], oracle_values = cpu_baseline(name, mesh, fmt, lam, mu)
        if main or name == "poisson2d":
            plan = cpu_plan_baselines(name, mesh, fmt, lam, mu)
            if "B5_sparsity" in plan:
                plan["B5_sparsity"]["gpu_structure_ms_once"] = structure_ms
            out["cpu_baseline"]["plan_baselines"] = plan

    # the opt-in minimal-instruction formulation, same mesh and steps
    ctx.formulation = fem.FORMULATION_MINIMAL
    t_min = time_assembly(fmt, ke, lam, mu, steps, 3, flush)
    ms_min = t_min["total_ms"] / steps
    roof_m, fp64_m = rooflines(ms_min, "minimal")
    mini = {"value": world * nnz / (ms_min * 1e-3), "ms_per_step": ms_min,
            "element_ms": statistics.mean(t_min["element_ms"]), "gather_ms": statistics.mean(t_min["gather_ms"]),
            "roofline_frac": roof_m["frac"], "fp64_roofline": fp64_m,
            "note": "AFEM_FORMULATION_MINIMAL: fewest FP64 instructions, closer to exact arithmetic than the "
                    "reference's formula, not bit-identical to it"}
    if oracle_values is not None:
        mini["max_rel_diff_vs_oracle"] = guard_error(fmt.values.cpu().numpy(), oracle_values, fmt.row_ptr.cpu().numpy(),
                                                     w["nb_dof"])
    out["minimal_formulation"] = mini
    ctx.formulation = fem.FORMULATION_REFERENCE
    fmt.element_matrices(ke, lam=lam, mu=mu)
    fmt.gather(ke)
    del ke, flush

    out["structure"] = time_structure(fmt)
    if not args.no_e2e:
        out["e2e"] = run_e2e(args, name, mesh, fmt, lam, mu)
    if not args.no_solve:
        out["solve"] = run_solve(args, name, ctx, mesh, fmt)
    return out


def run_gpu(args):
    import torch
    import torch.distributed as dist

    from arcanefem_gb300 import fem

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    ctx = fem.Context()
    main = measure_workload(args, args.workload, args.n, ctx, rank, world, local, main=True)
    extras = {}
    if not args.no_extra_workloads:
        for name in EXTRA_WORKLOADS:
            if name != args.workload:
                extras[name] = measure_workload(args, name, WORKLOADS[name]["n"], ctx, rank, world, local, main=False)
    learned = None if (args.no_learned or rank != 0) else run_learned(args)
    batched = None if (args.no_batched or rank != 0) else run_batched(args)

    if rank == 0:
        w = WORKLOADS[args.workload]
        out = {
            "metric": w["metric"], "value": main.pop("value"), "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": max(args.warmup, 3), "ms_per_step": main.pop("ms_per_step"), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered mesh)",
            "config": main.pop("config"), "gpu_launches": main.pop("gpu_launches"), "clocks": main.pop("clocks"),
        }
        main.pop("unit")
        out.update(main)
        for v in extras.values():
            v["metric"] = "assembled nnz/s"
        out["workloads"] = extras
        out["learned"] = learned
        out["batched"] = batched
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_e2e(args, name, mesh, fmt0, lam, mu):
    """Same metric through the public API with host buffers (transfers timed).

    The step of the headline metric reuses the sparsity, so the e2e step does
    too: the node coordinates go host -> device, the element matrices and the
    node-wise gather run through the API, and the values come back device ->
    host, every step.  ``rebuild`` times the from-scratch path as well: the
    mesh (coordinates and cells) host -> device, node -> cell, sparsity,
    assembly, and the whole block CSR back."""
    import torch

    from arcanefem_gb300 import fem

    w = WORKLOADS[name]
    nnz = fmt0.nnzb * w["nb_dof"] ** 2
    coords_h = torch.from_numpy(mesh.coords).pin_memory()
    cells_h = torch.from_numpy(mesh.cells).pin_memory()
    vals_h = torch.empty(nnz, dtype=torch.float64).pin_memory()
    cols_h = torch.empty(fmt0.nnzb, dtype=torch.int32).pin_memory()
    rp_h = torch.empty(mesh.nb_node + 1, dtype=torch.int32).pin_memory()
    ctx = fem.Context()
    dco = torch.empty_like(coords_h, device="cuda")
    dce = torch.empty_like(cells_h, device="cuda")
    ke = torch.empty(fmt0.element_buffer_size(), dtype=torch.float64, device="cuda")
    steps = max(3, args.steps // 2)
    chunks = args.e2e_chunks   # 0: the library's choice, one range per ~80 MB of values

    def timed(one, blocks=3):
        """Median over `blocks` timed blocks of `steps` steps (host-synchronised
        steps: the median keeps one disturbed block from setting the figure)."""
        for _ in range(2):
            one()
        per = []
        for _ in range(blocks):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(steps):
                one()
            torch.cuda.synchronize()
            per.append((time.perf_counter() - t0) / steps)
        return statistics.median(per)

    # values step: structure built once, as the reference module does at init
    dco.copy_(coords_h)
    dce.copy_(cells_h)
    fs = fem.BSRFormat(ctx, fem.Mesh(mesh.dim, dco, dce))
    fs.initialize(w["nb_dof"])
    fs.compute_sparsity()

    def values_step():   # host coordinates in, in node prefixes; cell ranges; values back behind them
        fs.assemble_to_host(ke, vals_h, chunks=chunks, lam=lam, mu=mu, coords_h=coords_h)



    side = torch.cuda.Stream()

    def rebuild_step():   # cells in; structure; its copy back on a side stream while the values assemble
        dce.copy_(cells_h, non_blocking=True)
        f = fem.BSRFormat(ctx, fem.Mesh(mesh.dim, dco, dce))
        f.initialize(w["nb_dof"])
        f.compute_sparsity()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            rp_h.copy_(f.row_ptr, non_blocking=True)
            cols_h.copy_(f.cols, non_blocking=True)
        f.assemble_to_host(ke, vals_h, chunks=chunks, lam=lam, mu=mu, coords_h=coords_h)
        side.synchronize()
        torch.cuda.current_stream().synchronize()

    dt = timed(values_step)
    assert torch.equal(vals_h, fmt0.values.cpu()), "host values differ from the device assembly's"
    dt_r = timed(rebuild_step)
    assert torch.equal(rp_h, fs.row_ptr.cpu()) and torch.equal(cols_h, fs.cols.cpu()), "rebuilt structure differs"
    assert torch.equal(vals_h, fmt0.values.cpu()), "rebuilt values differ"
    # the coordinates do come from the host in every step: with the device copy
    # poisoned, one more step of each kind still gives the same values
    dco.fill_(float("nan"))
    vals_h.fill_(0.0)
    values_step()
    assert torch.equal(vals_h, fmt0.values.cpu()), "values step did not upload the coordinates"
    dco.fill_(float("nan"))
    vals_h.fill_(0.0)
    rebuild_step()
    assert torch.equal(vals_h, fmt0.values.cpu()), "rebuild step did not upload the coordinates"
    h2d = coords_h.numel() * 8
    d2h = nnz * 8
    return {"value": nnz / dt, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": dt * 1e3, "steps": steps, "timing": f"median of 3 wall-clock blocks of {steps} steps",
            "includes": ("H2D node coordinates in node prefixes, each ahead of the cell range that first uses it, "
                         "element matrices and gather in cell ranges, each completed node range's values D2H behind "
                         f"it ({chunks or 'auto: one per ~80 MB of values, max 12'} ranges; sparsity reused)"),
            "rebuild": {"value": nnz / dt_r, "unit": UNIT, "ms_per_step": dt_r * 1e3,
                        "h2d_bytes_per_step": h2d + cells_h.numel() * 4,
                        "d2h_bytes_per_step": d2h + fmt0.nnzb * 4 + (mesh.nb_node + 1) * 4,
                        "includes": ("H2D cells, node->cell, sparsity; then the row pointers and columns D2H on a "
                                     "side stream while the values assemble as in the values step (coordinates "
                                     "H2D in node prefixes, values D2H behind the node ranges)")}}


def oracle_kind(name):
    from oracle import oracle as O
    w = WORKLOADS[name]
    if w["nb_dof"] == 3:
        return O.ELASTICITY_TET4
    if w.get("cell") == "hex":
        return O.POISSON_HEXA8
    return O.POISSON_TET4 if w["dim"] == 3 else O.POISSON_TRI3


def guard_error(got, ref, rp, b):
    """max |got - ref| / max(|ref|, 1e-3 max|row|) per (block) row: the parity
    tests' guard for the minimal formulation."""
    import numpy as np
    row_of = np.repeat(np.arange(rp.size - 1), np.diff(rp) * b * b)
    rowmax = np.zeros(rp.size - 1)
    np.maximum.at(rowmax, row_of, np.abs(ref))
    return float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), np.where(rowmax[row_of] > 0,
                                                                             1e-3 * rowmax[row_of], 1.0))))


def cpu_baseline(name, mesh, fmt, lam, mu):
    """The oracle's node-wise assembly (CPU restatement of BSRFormat.h:473-537 with
    the reference element vectors) on all host cores, same mesh and sparsity,
    and the GPU values compared with it entry by entry."""
    import numpy as np

    from oracle import oracle as O

    threads = O.max_threads()
    ptr, nc = fmt.nc_ptr.cpu().numpy(), fmt.nc_cell.cpu().numpy()
    rp, cols = fmt.row_ptr.cpu().numpy(), fmt.cols.cpu().numpy()
    b = WORKLOADS[name]["nb_dof"]
    nnz = fmt.nnzb * b * b
    t0 = time.perf_counter()
    v = O.assemble(oracle_kind(name), mesh.coords, mesh.cells, ptr, nc, rp, cols, lam=lam, mu=mu, nb_threads=threads)
    dt = time.perf_counter() - t0
    gpu = fmt.values.cpu().numpy()
    return {"value": nnz / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"one full values assembly of the same mesh ({mesh.nb_cell} cells), {dt:.2f} s",
            "bit_exact_vs_gpu": bool(np.array_equal(gpu, v)),
            "entries_differing_from_gpu": int(np.count_nonzero(gpu != v)),
            "max_rel_diff_vs_gpu": guard_error(gpu, v, rp, b)}, v


def cpu_plan_baselines(name, mesh, fmt, lam, mu, budget_s=5.0):
    """The CPU baselines of the plan beside the all-core node-wise assembly:
    B1 the reference's DOK assembly (ordered map, zeros skipped; Poisson only),
    1 core, on the first cells that fit the budget, scaled to the whole mesh;
    B2 the node-wise assembly on 1 core; B5 the sparsity build, node-wise on
    all cores and edge-sort on 1 core."""
    from oracle import oracle as O

    w = WORKLOADS[name]
    b = w["nb_dof"]
    nnz = fmt.nnzb * b * b
    threads = O.max_threads()
    ptr, nc = fmt.nc_ptr.cpu().numpy(), fmt.nc_cell.cpu().numpy()
    rp, cols = fmt.row_ptr.cpu().numpy(), fmt.cols.cpu().numpy()
    out = {}
    if b == 1 and w.get("cell") != "hex":
        kind = oracle_kind(name)
        probe = min(mesh.nb_cell, 20000)
        t0 = time.perf_counter()
        O.assemble_dok(kind, mesh.nb_node, mesh.coords, mesh.cells, nb_cell=probe)
        per_cell = (time.perf_counter() - t0) / probe
        sample = int(min(mesh.nb_cell, max(probe, budget_s / max(per_cell, 1e-9))))
        t0 = time.perf_counter()
        O.assemble_dok(kind, mesh.nb_node, mesh.coords, mesh.cells, nb_cell=sample)
        dt = time.perf_counter() - t0
        est = dt * mesh.nb_cell / sample
        out["B1_dok_1core"] = {"value": nnz / est, "unit": UNIT, "cores": 1, "kind": "port",
                               "estimated_full_s": est,
                               "sample": f"the first {sample} of {mesh.nb_cell} cells into the ordered map, {dt:.2f} s, "
                                         "scaled by the cell count"}
    t0 = time.perf_counter()
    O.assemble(oracle_kind(name), mesh.coords, mesh.cells, ptr, nc, rp, cols, lam=lam, mu=mu, nb_threads=1)
    dt = time.perf_counter() - t0
    out["B2_nodewise_1core"] = {"value": nnz / dt, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": f"one full values assembly, {dt:.2f} s"}
    if b == 1:
        t0 = time.perf_counter()
        O.sparsity_nodewise(mesh.nb_node, mesh.cells, ptr, nc, nb_threads=threads)
        t_nw = time.perf_counter() - t0
        t0 = time.perf_counter()
        O.sparsity(mesh.nb_node, mesh.cells)
        t_es = time.perf_counter() - t0
        out["B5_sparsity"] = {"nodewise_all_cores_ms": t_nw * 1e3, "cores": threads,
                              "edge_sort_1core_ms": t_es * 1e3, "kind": "port",
                              "gpu_structure_ms_once": None}
    return out


def run_solve(args, name, ctx, mesh, fmt):
    """Time to the target relative residual on the assembled system (RowColumn
    elimination Dirichlet, source / body force), FP64 CG and mixed precision."""
    import torch

    from arcanefem_gb300 import fem

    w = WORKLOADS[name]
    nd = mesh.nb_node * w["nb_dof"]
    nodes = torch.as_tensor(mesh.groups[w["dirichlet"]], device="cuda")
    res = {"target_relres": w["rtol"], "dirichlet": f"row-column elimination on {w['dirichlet']}"}
    x_oracle = None
    for prec in ("fp64", "mixed"):
        # re-assemble: the transformation of the previous solve modified the values in place
        ke = torch.empty(fmt.element_buffer_size(), dtype=torch.float64, device="cuda")
        lam, mu = fem.lame(w["E"], w["nu"]) if w["nb_dof"] == 3 else (0.0, 0.0)
        fmt.element_matrices(ke, lam=lam, mu=mu)
        fmt.gather(ke)
        del ke
        ls = fem.DoFLinearSystem(ctx, nd)
        fmt.to_linear_system(ls)
        # the right-hand side and the boundary conditions, timed on the device
        # (the second, warm application is the one reported)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        t_bc = time.perf_counter()
        ev[0].record()
        if w["nb_dof"] == 3:
            fmt.rhs_body_force(w["body"], ls.rhs_variable())
            for comp in range(3):
                ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, nodes, 3, comp, 0.0)
        else:
            fmt.rhs_constant_source(w["source"], ls.rhs_variable())
            ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, nodes, 1, 0, 0.0)
        ls.apply_matrix_transformation()
        ls.apply_rhs_transformation()
        ev[1].record()
        torch.cuda.synchronize()
        nnz_s = fmt.nnzb * w["nb_dof"] ** 2
        # one pass over the matrix (columns, values) and the vectors (rhs, flags, values of the forced DoFs)
        bc_bytes = 12 * nnz_s + 4 * (nd + 1) + 8 * nd + 2 * nd + 8 * nd
        bc_ms = ev[0].elapsed_time(ev[1])
        res["bc"] = {"device_ms": bc_ms, "wall_ms": (time.perf_counter() - t_bc) * 1e3,
                     "steps": "source RHS, Dirichlet flags, applyMatrixTransformation, applyRHSTransformation",
                     "one_pass_bytes": bc_bytes, "achieved_gbs": bc_bytes / (bc_ms * 1e-3) / 1e9,
                     "frac_of_hbm": bc_bytes / (bc_ms * 1e-3) / 1e9 / read_peaks()[0]}
        opt = fem.solver_options(rtol=w["rtol"], max_iter=20000,
                                 precision=fem.PRECISION_MIXED if prec == "mixed" else fem.PRECISION_FP64,
                                 inner_rtol=args.inner_rtol)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        info = ls.solve(opt)
        torch.cuda.synchronize()
        wall = (time.perf_counter() - t0) * 1e3
        res[prec] = {"solve_ms": info.solve_ms, "wall_ms": wall, "iterations": info.iterations,
                     "refinements": info.refinements, "true_relres": info.relres, "status": info.status}
        x = ls.solution_variable()
        if prec == "fp64":
            x_fp64 = x.clone()
            if not args.no_cpu_baseline:
                res["cpu_fp64_cg"], x_oracle = cpu_solve_baseline(fmt, ls, info.iterations, w["rtol"])
        else:   # error against the FP64 CG solution of the same system
            res[prec]["error_vs_fp64_cg"] = float(torch.linalg.norm(x - x_fp64) / torch.linalg.norm(x_fp64))
        if x_oracle is not None:   # error against the oracle's FP64 solution to the same target
            xo = torch.as_tensor(x_oracle)
            res[prec]["error_vs_oracle"] = float(torch.linalg.norm(x.cpu() - xo) / torch.linalg.norm(xo))
        ls.close()
    return res


def cpu_solve_baseline(fmt, ls, gpu_iterations, rtol, cap=300, budget_s=20.0):
    """The oracle's Jacobi PCG (CPU restatement of the reference's diagonal-
    preconditioned CG) on the same transformed system, all host cores, for at
    most `cap` iterations; the time to the target is that rate times the GPU
    solver's iteration count (the two run the same iteration).  When that
    estimate fits in `budget_s`, the oracle then solves to the same target
    from zero as well: its measured time, and its solution (returned second,
    else None) against which each GPU solution's error is reported."""
    from oracle import oracle as O

    rp, cols, vals = (t.cpu().numpy() for t in fmt.to_csr())
    b = ls.rhs_variable().cpu().numpy()
    threads = O.max_threads()
    iters = int(min(gpu_iterations, cap))
    t0 = time.perf_counter()
    _, it, rel = O.pcg_jacobi(rp, cols, vals, b, rtol=1e-300, max_iter=iters, nb_threads=threads)
    dt = time.perf_counter() - t0
    per_it = dt / max(it, 1)
    t0 = time.perf_counter()
    _, it1, _ = O.pcg_jacobi(rp, cols, vals, b, rtol=1e-300, max_iter=min(iters, 50), nb_threads=1)
    per_it1 = (time.perf_counter() - t0) / max(it1, 1)
    out = {"ms_per_iteration": per_it * 1e3, "iterations_sampled": it, "cores": threads, "kind": "port",
           "estimated_solve_ms": per_it * gpu_iterations * 1e3,
           "sample": f"{it} Jacobi-PCG iterations on the same system, {dt:.2f} s",
           "B4_1core": {"ms_per_iteration": per_it1 * 1e3, "estimated_solve_ms": per_it1 * gpu_iterations * 1e3,
                        "cores": 1, "sample": f"{it1} iterations"}}
    x_oracle = None
    if per_it * gpu_iterations <= budget_s:
        t0 = time.perf_counter()
        x_oracle, it2, rel2 = O.pcg_jacobi(rp, cols, vals, b, rtol=rtol, max_iter=20000, nb_threads=threads)
        out["full_solve"] = {"solve_ms": (time.perf_counter() - t0) * 1e3, "iterations": it2, "relres": rel2}
    return out, x_oracle


def run_learned(args):
    """Variable-coefficient diffusion on a 512^2 triangle grid (k = exp(GRF),
    correlation 0.05, variance 1; bump source; u = 0 on the boundary): time to
    a 1e-8 FP64 relative residual of plain FP64 CG (Jacobi and none) against
    flexible CG with the learned V-cycle preconditioner (M in FP32, network
    BF16), trained on 2000 solver-generated pairs.  Device time per solve
    (CUDA events); training and pair generation reported separately."""
    import numpy as np
    import torch

    from arcanefem_gb300 import fem, learned

    n = args.learned_n
    levels = int(np.log2(n)) if n >= 8 else 3
    ctx = fem.Context()
    t0 = time.perf_counter()
    prob, hier, net = learned.setup(ctx, n=n, levels=levels, layers=6, seed=7, max_batch=16)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    b = prob.rhs(np.random.default_rng(123))

    sols = {}

    def best(fn, reps=3, tag=None):
        out = [fn() for _ in range(reps)]
        info, x = min(out, key=lambda o: o[0].solve_ms)
        if tag:
            sols[tag] = x
        return info

    def cg(precond):
        x = torch.zeros_like(b)
        info = fem.cg_solve_csr(ctx, prob.row_ptr, prob.cols, prob.values, b, x,
                                options=fem.solver_options(rtol=1e-8, max_iter=50000, precond=precond))
        return info, x

    def fcg():
        x = torch.zeros_like(b)
        return net.fcg(prob.row_ptr, prob.cols, prob.values, b, x, fem.solver_options(rtol=1e-8, max_iter=5000)), x

    cg_jac = best(lambda: cg(fem.PRECOND_JACOBI), 2, tag="fp64")
    cg_none = best(lambda: cg(fem.PRECOND_NONE), 1)
    untrained = best(fcg, tag="untrained")
    t0 = time.perf_counter()
    R, E = learned.make_training_pairs(prob, count=2000, solves=20, every=25, seed=4)
    torch.cuda.synchronize()
    pairs_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    rep = learned.train_validated(net, prob, R, E, prob.rhs(np.random.default_rng(77)), epochs=4, batch=16, lr=2e-3)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    kept = best(fcg, tag="learned")
    net.close()

    def err(tag):   # relative error against the FP64 Jacobi-CG solution of the same system
        return float(torch.linalg.norm(sols[tag] - sols["fp64"]) / torch.linalg.norm(sols["fp64"]))

    oracle_solve = None
    if not args.no_cpu_baseline:   # the oracle's FP64 Jacobi PCG to the same target, all host cores
        from oracle import oracle as O
        t0 = time.perf_counter()
        xo, it_o, rel_o = O.pcg_jacobi(prob.row_ptr.cpu().numpy(), prob.cols.cpu().numpy(),
                                        prob.values.cpu().numpy(), b.cpu().numpy(), rtol=1e-8, max_iter=50000,
                                        nb_threads=O.max_threads())
        xo = torch.as_tensor(xo)
        oracle_solve = {"solve_ms": (time.perf_counter() - t0) * 1e3, "iterations": it_o, "relres": rel_o,
                        "cores": O.max_threads(), "kind": "port",
                        "error_vs_oracle": {t: float(torch.linalg.norm(sols[t].cpu() - xo) / torch.linalg.norm(xo))
                                            for t in ("fp64", "untrained", "learned")}}

    def d(info):
        return {"solve_ms": info.solve_ms, "iterations": info.iterations, "true_relres": info.relres,
                "status": info.status}
    return {
        "problem": f"-div(k grad u) = f, {n}^2 quads x 2 triangles ({2 * n * n} tris), k = exp(GRF 0.05, var 1)",
        "target_relres": 1e-8,
        "plain_fp64_cg_jacobi": d(cg_jac), "plain_fp64_cg_none": d(cg_none),
        "fcg_vcycle_untrained": dict(d(untrained), error_vs_fp64_cg=err("untrained")),
        "fcg_learned": dict(d(kept), error_vs_fp64_cg=err("learned")),
        "cpu_oracle_fp64_cg_jacobi": oracle_solve,
        "speedup_vs_plain_fp64_cg_jacobi": cg_jac.solve_ms / kept.solve_ms,
        "speedup_vs_plain_fp64_cg_none": cg_none.solve_ms / kept.solve_ms,
        "network": ("6 message-passing layers, width 64, BF16 tcgen05 GEMMs (TMA-fed, FP32 accumulate in TMEM); predicts the "
                    "smoothers of a V(1,1)-cycle on a 9-level Galerkin hierarchy: per-node weights, and factored sparse "
                    "approximate inverses theta L^T L (edge heads) on the finest and the coarse levels"),
        "training": {"pairs": 2000, "pair_generation_s": pairs_s, "train_s": train_s, "loss": rep["loss"],
                     "fcg_iterations_untrained": rep["iterations_untrained"],
                     "fcg_iterations_trained": rep["iterations_trained"], "kept": rep["kept"]},
        "setup_s": setup_s,
    }


def run_batched(args):
    """64 Poisson instances (sides N ~ U{64..512}, seeded), 4 bump right-hand
    sides each, assembled and solved to a 1e-8 FP64 relative residual in one
    persistent cooperative launch (CUDA graph), autotuned; against the same
    systems solved one right-hand side at a time through the single-system
    FP64 CG."""
    import numpy as np
    import torch

    from arcanefem_gb300 import batch as B
    from arcanefem_gb300 import fem

    ctx = fem.Context()
    sizes = B.instance_sizes(args.batched_count, args.batched_sides[0], args.batched_sides[1], seed=2024)
    t0 = time.perf_counter()
    bt = B.Batch(ctx, sizes, seed=7)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    opt = fem.solver_options(rtol=1e-8, inner_rtol=0.1, max_iter=20000)
    t0 = time.perf_counter()
    cands = [(128, 8, 3.0), (128, 8, 3.5), (256, 4, 3.0), (256, 4, 3.5), (256, 3, 3.5), (512, 2, 3.5)]
    tune = (bt.autotune(candidates=cands, options=opt, reps=1) if args.batched_tune == "auto"
            else {"cached": False, "config": {}})
    tune_s = time.perf_counter() - t0
    runs = [bt.solve(opt) for _ in range(3)]
    res, ms = min(runs, key=lambda r: r[1])
    # the same systems through the single-system API: FP64 CG, first right-hand side of every instance
    single_ms = 0.0
    for i in range(len(sizes)):
        f = bt.fmts[i]
        bi = bt.rhs[i][:, 0].contiguous()
        x = torch.zeros_like(bi)
        info = fem.cg_solve_csr(ctx, f.row_ptr, f.cols, f.values, bi, x,
                                options=fem.solver_options(rtol=1e-8, max_iter=50000))
        single_ms += info.solve_ms
    cfg, grid = bt.config()
    dofs = bt.nb_node * B.RHS
    fin = [r.finish_ms for r in res]
    out = {
        "instances": len(sizes), "sides": [min(sizes), max(sizes)], "nodes": bt.nb_node, "nnz": bt.nnz,
        "rhs_per_instance": B.RHS, "target_relres": 1e-8,
        "batch_ms": ms, "dof_rhs_per_s": dofs / (ms * 1e-3),
        "max_relres": max(max(r.relres) for r in res),
        "inner_iterations_max": max(r.inner_iterations for r in res),
        "refinements_max": max(r.refinements for r in res),
        "team_finish_ms": {"min": min(fin), "median": float(np.median(fin)), "max": max(fin)},
        "config": {**cfg.as_dict(), "grid_ctas": grid, "rebalanced": tune["config"].get("weights") is not None,
                   "from_cache": tune["cached"],
                   "team_finish_spread_ms": tune["config"].get("team_finish_spread")},
        "autotune_s": tune_s, "setup_s": setup_s,
        "single_system_fp64_cg_ms_one_rhs": single_ms,
        "speedup_vs_single_system_4_rhs": 4 * single_ms / ms,
        "launches_per_batch": 1,
    }
    bt.close()
    return out


# ---------------------------------------------------------------------------
def run_reference(args):
    """CPU reference arm: the oracle's restatement of the reference node-wise
    assembly on all host threads, rank 0 only."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from arcanefem_gb300 import fem
    from oracle import oracle as O

    w = WORKLOADS[args.workload]
    mesh = make_mesh(args.workload, args.n, args.seed)
    ptr, nc, _ = O.node_cell(mesh.nb_node, mesh.cells)
    rp, cols = O.sparsity(mesh.nb_node, mesh.cells)
    nnz = int(rp[-1]) * w["nb_dof"] ** 2
    lam, mu = fem.lame(w["E"], w["nu"]) if w["nb_dof"] == 3 else (0.0, 0.0)
    threads = O.max_threads()
    kind = oracle_kind(args.workload)
    for _ in range(args.warmup):
        O.assemble(kind, mesh.coords, mesh.cells, ptr, nc, rp, cols, lam=lam, mu=mu, nb_threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        O.assemble(kind, mesh.coords, mesh.cells, ptr, nc, rp, cols, lam=lam, mu=mu, nb_threads=threads)
        times.append(time.perf_counter() - t0)
    ms = 1e3 * sum(times) / len(times)
    value = nnz / (ms * 1e-3)
    out = {"metric": w["metric"], "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded jittered mesh)",
           "config": config(args.workload, args.n, args.seed, 1), "impl": "reference",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"full values assembly of the same mesh per step ({mesh.nb_cell} cells)"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "ArcaneFEM needs Arcane/.NET/MPI/HYPRE, absent here: CPU restatement of its node-wise assembly"}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    a = parse_args()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_gpu(a)
