"""The allocation-free assembly entry point, for callers that cannot let the
library allocate device memory (a framework that owns and budgets every
device allocation through its own pool, or a step loop that cannot afford
the synchronisation a device allocation implies).

afem_assemble_poisson_p1_noalloc keeps its element rows in a fixed device
array inside the library instead of a context's scratch arena.  This test
calls it through the C ABI, twice in a row on two different meshes (the
second call reuses the array left by the first), and compares each result
with the regular afem_assemble_poisson_p1 on the same inputs, within the
1e-12 per-entry tolerance of the other parity tests.  It also checks that a
mesh above the array's size is refused with AFEM_ERR_BAD_ARG.  Kept in its
own file so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from arcanefem_gb300 import _capi, fem, meshgen

pytestmark = pytest.mark.gpu


def _format(ctx, mesh):
    f = fem.BSRFormat(ctx, fem.Mesh.from_host(mesh.dim, mesh.coords, mesh.cells))
    f.initialize(1)
    f.compute_sparsity()
    return f


def _noalloc(f, values, coeff=None):
    mv = f.mesh_view()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    return _capi.lib().afem_assemble_poisson_p1_noalloc(stream, C.byref(mv), C.c_void_p(f.row_ptr.data_ptr()),
                                                         C.c_void_p(0 if coeff is None else coeff.data_ptr()),
                                                         C.c_void_p(values.data_ptr()))


def _rel(got, ref, rp):
    row_of = np.repeat(np.arange(rp.size - 1), np.diff(rp))
    rowmax = np.zeros(rp.size - 1)
    np.maximum.at(rowmax, row_of, np.abs(ref))
    return float(np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-3 * rowmax[row_of])))


def test_noalloc_matches_regular_assembly_two_calls_in_a_row():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = fem.Context()
    try:
        meshes = [meshgen.unit_cube_tet(12, seed=21), meshgen.unit_square_tri(150, seed=22)]
        coeffs = [None, torch.as_tensor(np.exp(np.random.default_rng(3).standard_normal(2 * 150 * 150)),
                                        device="cuda")]
        for mesh, coeff in zip(meshes, coeffs):
            f = _format(ctx, mesh)
            f.assemble_poisson(coeff)                      # regular entry point (context scratch)
            ref = f.values.cpu().numpy()
            rp = f.row_ptr.cpu().numpy()
            out = torch.full_like(f.values, float("nan"))
            assert _noalloc(f, out, coeff) == 0, _capi.lib().afem_last_error()
            torch.cuda.synchronize()
            assert _rel(out.cpu().numpy(), ref, rp) < 1e-12
    finally:
        ctx.close()


def test_noalloc_refuses_meshes_above_its_fixed_size():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    ctx = fem.Context()
    try:
        f = _format(ctx, meshgen.unit_cube_tet(36, jitter=0.0))    # 279,936 tetrahedra > 262,144
        out = torch.zeros_like(f.values)
        assert _noalloc(f, out) == _capi.AFEM_OK + 1                 # AFEM_ERR_BAD_ARG
        assert b"262144 tetrahedra" in _capi.lib().afem_last_error()
        assert float(out.abs().max()) == 0.0                        # nothing was launched
    finally:
        ctx.close()
