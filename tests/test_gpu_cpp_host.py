"""The C++ host mirror (include/afem_gb300.hpp) drives the same GPU path:
the example program's solution equals the Python-API solution."""
import os
import subprocess

import numpy as np
import pytest
import torch

from arcanefem_gb300 import fem, meshgen

pytestmark = pytest.mark.gpu

EXE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "arcanefem_gb300", "lib",
                   "poisson_cube")


def test_cpp_host_example_matches_python_api(cuda_ctx, tmp_path):
    if not os.path.exists(EXE):
        from arcanefem_gb300 import build
        build.build()
    n = 8
    out = tmp_path / "u.bin"
    r = subprocess.run([EXE, str(n), str(out)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "eliminate_row_throws=1" in r.stdout
    u_cpp = np.fromfile(out, dtype=np.float64)
    m = meshgen.unit_cube_tet(n, jitter=0.0)
    dm = fem.Mesh.from_host(3, m.coords, m.cells)
    f = fem.BSRFormat(cuda_ctx, dm)
    f.initialize(1)
    f.compute_sparsity()
    f.assemble_poisson()
    ls = fem.DoFLinearSystem(cuda_ctx, m.nb_node)
    f.to_linear_system(ls)
    f.rhs_constant_source(1.0, ls.rhs_variable())
    ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, torch.as_tensor(m.groups["x_faces"], device="cuda"), 1,
                                   0, 0.0)
    ls.apply_linear_system_transformation_and_solve(fem.solver_options(rtol=1e-10, max_iter=10000))
    u_py = ls.solution_variable().cpu().numpy()
    assert u_cpp.shape == u_py.shape
    assert np.max(np.abs(u_cpp - u_py)) <= 1e-9 * np.max(np.abs(u_py))
