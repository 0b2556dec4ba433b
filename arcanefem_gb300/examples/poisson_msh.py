"""Poisson on a gmsh mesh, end to end on the GPU, solution written as VTU.

    python -m arcanefem_gb300.examples.poisson_msh mesh.msh out.vtu \\
        --f 5.5 --dirichlet boundary=0.5 [--neumann top=1.0]

The Poisson module's steps (modules/poisson/FemModule.cc:163-196): node-wise
assembly of the stiffness, constant source, Neumann flux on named face
groups, Dirichlet values on named node groups (penalty by default, as the
module), CG to rtol, then the solution is written with the mesh for ParaView.
"""
from __future__ import annotations

import argparse

import numpy as np
import torch

from arcanefem_gb300 import fem, meshio


def solve(path: str, f: float, dirichlet: dict, neumann: dict | None = None, rtol: float = 1e-10,
          ctx: fem.Context | None = None, method: str = "penalty", penalty: float = 1e30):
    """method: "penalty" (the reference's default, FemBoundaryConditions.axl)
    or "rowcolumn" (RowColumnElimination, with the reference's column_index > 0
    test, which keeps column 0: for a non-zero value on node 0 the system is
    then not symmetric)."""
    d = meshio.read_msh(path)
    m = d.mesh
    ctx = ctx or fem.Context()
    fmt = fem.BSRFormat(ctx, fem.Mesh.from_host(m.dim, m.coords, m.cells))
    fmt.initialize(1)
    fmt.compute_sparsity()
    fmt.assemble_poisson()
    ls = fem.DoFLinearSystem(ctx, m.nb_node)
    fmt.to_linear_system(ls)
    fmt.rhs_constant_source(f, ls.rhs_variable())
    for name, g in (neumann or {}).items():
        faces, outward = d.faces[name]
        fem.rhs_boundary_faces(ctx, m.dim, fmt.mesh.coords, torch.as_tensor(faces, device="cuda"),
                               torch.as_tensor(outward, device="cuda"), fem.FACE_SCALAR, [g], 1, ls.rhs_variable())
    for name, value in dirichlet.items():
        nodes = torch.as_tensor(m.groups[name], device="cuda")
        if method == "penalty":
            ls.apply_dirichlet_penalty(nodes, 1, 0, float(value), penalty)
        else:
            ls.apply_dirichlet_elimination(fem.ELIMINATE_ROW_COLUMN, nodes, 1, 0, float(value))
    info = ls.apply_linear_system_transformation_and_solve(
        fem.solver_options(rtol=rtol, max_iter=100000, skip_forced_rows=method == "penalty"))
    u = ls.solution_variable().cpu().numpy().copy()
    ls.close()
    return d, u, info


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("mesh")
    p.add_argument("out")
    p.add_argument("--f", type=float, default=1.0)
    p.add_argument("--dirichlet", action="append", default=[], help="group=value")
    p.add_argument("--neumann", action="append", default=[], help="face_group=flux")
    p.add_argument("--rtol", type=float, default=1e-10)
    p.add_argument("--method", choices=["penalty", "rowcolumn"], default="penalty")
    a = p.parse_args(argv)
    dirichlet = {k: float(v) for k, v in (s.split("=") for s in a.dirichlet)}
    neumann = {k: float(v) for k, v in (s.split("=") for s in a.neumann)}
    d, u, info = solve(a.mesh, a.f, dirichlet, neumann, a.rtol, method=a.method)
    meshio.write_vtu(a.out, d.mesh, point_data={"U": u}, cell_data={"cell_id": np.arange(d.mesh.nb_cell)})
    print(f"{a.mesh}: {d.mesh.nb_node} nodes, {d.mesh.nb_cell} cells; CG {info.iterations} iterations, "
          f"relres {info.relres:.2e} -> {a.out}")


if __name__ == "__main__":
    main()
