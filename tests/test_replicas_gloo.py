"""bench.py's multi-GPU form is replicas only: each rank assembles its own
copy, the job time is the max over ranks, rank 0 alone reports, and the CPU
reference arm runs on rank 0 only.  Exercised with two gloo ranks on CPU,
each assembling a small mesh with the oracle."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench
    from arcanefem_gb300 import meshgen
    from oracle import oracle as O
    dist.init_process_group("gloo", rank=rank, world_size=world)
    m = meshgen.unit_square_tri(16 + 8 * rank, seed=rank)
    ptr, nc, _ = O.node_cell(m.nb_node, m.cells)
    rp, cols = O.sparsity(m.nb_node, m.cells)
    v = O.assemble(O.POISSON_TRI3, m.coords, m.cells, ptr, nc, rp, cols)
    assert v.size == rp[-1]
    local_ms = 10.0 * (rank + 1)          # rank 1 is the slow replica
    ms, value = bench.replica_value(local_ms, world, 1000, 2, "cpu")
    out.put((rank, ms, value))
    dist.destroy_process_group()


def test_two_gloo_replicas_take_the_max_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, ms, value in got:
        assert ms == pytest.approx(10.0)          # max(10, 20) ms over 2 steps
        assert value == pytest.approx(2 * 1000 / 10e-3)


def test_reference_arm_reports_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "poisson2d", "--n", "16", "--steps", "1", "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_line_on_rank_zero():
    import json
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "poisson2d", "--n", "16", "--steps", "2", "--warmup", "1"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["cores"] >= 1
