"""The Arcane linear-system service (arcanefem_gb300/arcane/GB300DoFLinearSystem.cc)
against the reference's interfaces.

CPU: the service compiles and links against stand-in headers that reproduce
the signatures of IDoFLinearSystemImpl, DoFLinearSystemImplBase,
IDoFLinearSystemFactory and CsrFormatMatrixView (tests/arcane_shim; Arcane
itself needs .NET, MPI and HYPRE, absent here).

GPU: a driver calls the service as a module does, with the reference's CSR
view as the assembly leaves it -- N row starts without a trailing entry and
unused (-1) slots inside rows -- on the device: set the view, apply the
matrix and right-hand-side transformations, solve; then clearValues and the
whole sequence again (a second solve).  Transformed values and right-hand
side: bit-exact against the oracle's transformations of the same system
without the unused slots; solutions: the oracle's Jacobi PCG solution within
1e-8 relative error, true residual below 1e-10.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

from arcanefem_gb300 import _capi, meshgen
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "tests", "arcane_shim")
ADAPTER = os.path.join(ROOT, "arcanefem_gb300", "arcane")


def cuda_home():
    from arcanefem_gb300 import build
    return os.path.dirname(os.path.dirname(os.path.realpath(build.nvcc())))


def build_driver(out_dir):
    if not os.path.exists(_capi.LIB_PATH):
        from arcanefem_gb300 import build
        build.build()
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    cuda = cuda_home()
    exe = os.path.join(str(out_dir), "adapter_driver")
    libdir = os.path.dirname(_capi.LIB_PATH)
    cmd = ["g++", "-O1", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
           "-I", SHIM, "-I", os.path.join(SHIM, "femutils"), "-I", ADAPTER, "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"),
           os.path.join(ADAPTER, "GB300DoFLinearSystem.cc"), os.path.join(SHIM, "adapter_driver.cc"),
           "-o", exe, "-L", libdir, "-lafem_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath," + libdir, "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return exe


def test_service_compiles_against_the_reference_interfaces(tmp_path):
    exe = build_driver(tmp_path)
    assert os.path.exists(exe)


def padded_view(rp, cols, vals, seed=0):
    """The reference CSR view of (rp, cols, vals): row starts only, plus
    unused (-1, value 0) slots scattered inside rows, as CsrFormat leaves
    slots it did not fill (femutils/CsrFormatMatrix.cc:49-50)."""
    rng = np.random.default_rng(seed)
    n = rp.size - 1
    rows, pc, pv, used = [], [], [], []
    for i in range(n):
        rows.append(len(pc))
        c = list(cols[rp[i]:rp[i + 1]])
        v = list(vals[rp[i]:rp[i + 1]])
        pos = list(range(len(c)))
        for _ in range(i % 3):
            k = int(rng.integers(0, len(c) + 1))
            c.insert(k, -1)
            v.insert(k, 0.0)
            pos = [p + (1 if p >= k else 0) for p in pos]
        base = len(pc)
        used.extend(base + p for p in pos)
        pc.extend(c)
        pv.extend(v)
    return (np.array(rows, np.int32), np.array(pc, np.int32), np.array(pv, np.float64), np.array(used, np.int64))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [0, 1])
def test_service_solves_a_padded_reference_view(cuda_ctx, tmp_path, precision):
    exe = build_driver(tmp_path)
    m = meshgen.unit_cube_tet(6, seed=11)
    n = m.nb_node
    ptr, nc, _ = O.node_cell(n, m.cells)
    rp, cols = O.sparsity(n, m.cells)
    vals = O.assemble(O.POISSON_TET4, m.coords, m.cells, ptr, nc, rp, cols)
    rhs = O.rhs_constant_source(3, m.coords, m.cells, ptr, nc, 1.0)
    fi = np.zeros(n, np.uint8)
    fv = np.zeros(n)
    ei = np.zeros(n, np.uint8)
    ev = np.zeros(n)
    # row-column elimination with a non-zero value on the x = 1 face, penalty on two interior nodes
    O.dirichlet_elimination(m.groups["x_max"] if "x_max" in m.groups else
                            np.flatnonzero(np.abs(m.coords[:, 0] - 1) < 1e-12).astype(np.int32),
                            1, 0, 0.5, O.ELIM_ROW_COLUMN, ei, ev)
    inner = np.flatnonzero((np.abs(m.coords[:, :3] - 0.5) < 0.2).all(1)).astype(np.int32)[:2]
    rhs_in = rhs.copy()
    O.dirichlet_penalty(inner, 1, 0, 0.2, 1e30, fi, fv, rhs_in)
    rows, pcols, pvals, used = padded_view(rp, cols, vals)
    d = tmp_path / "in"
    d.mkdir()
    (d / "meta.txt").write_text(f"{n} {pcols.size} {precision}\n")
    for name, a in (("rows.i32", rows), ("cols.i32", pcols), ("vals.f64", pvals), ("rhs.f64", rhs_in),
                    ("forced_info.u8", fi), ("forced_value.f64", fv), ("elim_info.u8", ei),
                    ("elim_value.f64", ev)):
        a.tofile(d / name)
    o = tmp_path / "out"
    o.mkdir()
    r = subprocess.run([exe, str(d), str(o)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    info = (o / "info.txt").read_text()
    assert "eliminateRow NotImplementedException" in info
    assert "matrixAddValue_outside FatalErrorException" in info and "done" in info
    # the oracle: the same transformations on the system without the unused slots
    tv, trhs = vals.copy(), rhs_in.copy()
    O.apply_transformations(rp, cols, tv, trhs, fi, fv, ei, ev)
    free = fi == 0   # the penalty rows stay out of both norms of the stop test (skip_forced_rows)
    xo, _, _ = O.pcg_jacobi(rp, cols, tv, trhs, rtol=1e-12, max_iter=20000, norm_skip=fi)
    unused = np.setdiff1d(np.arange(pcols.size), used)
    for p in (1, 2):
        got_v = np.fromfile(o / f"values{p}.f64")
        assert np.array_equal(got_v[used], tv), f"pass {p}: transformed values differ"
        assert np.all(got_v[unused] == 0.0), f"pass {p}: an unused slot was written"
        assert np.array_equal(np.fromfile(o / f"rhs{p}.f64"), trhs), f"pass {p}: transformed rhs differs"
        x = np.fromfile(o / f"sol{p}.f64")
        assert np.linalg.norm(x - xo) <= 1e-8 * np.linalg.norm(xo), f"pass {p}"
        res = np.linalg.norm((trhs - O.spmv(rp, cols, tv, x))[free]) / np.linalg.norm(trhs[free])
        assert res < 1e-10, (p, res)
        assert f"pass {p} iterations" in info and "status 0" in info
