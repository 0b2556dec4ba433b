"""Generate the golden fixtures that pin the CPU oracle.

Run once, in a checkout next to the ArcaneFEM sources:

    python tests/golden/make_fixtures.py /path/to/arcanefem

It reads the reference's own test meshes (binary gmsh 4.1) and solution check
files, and writes one compact ``.npz`` per case into this folder.  The tests
only read the ``.npz`` files, so the ArcaneFEM tree is not needed at test
time.  Each case records the mesh, the Dirichlet node sets (by physical
group name) and the reference solution (node uid -> value(s)) together with
the case parameters taken from the reference's ``.arc`` input.
"""
from __future__ import annotations

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
from arcanefem_gb300 import meshio  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))

# case name -> (mesh, check file, parameters).  Parameters restate the .arc inputs.
CASES = {
    # modules/testlab/inputs/Test.L-shape.2D.nwcsr.arc
    "testlab_lshape_2d": dict(
        mesh="meshes/msh/L-shape.msh", check="modules/testlab/tests/poisson_test_ref_L-shape_2D.txt",
        kind="testlab", f=-5.5, dirichlet=[("boundary", 0.5)], penalty=1e30, eps=1e-4, min_value=1e-16),
    # modules/testlab/inputs/Test.L-shape.3D.nwcsr.arc
    "testlab_lshape_3d": dict(
        mesh="meshes/msh/L-shape-3D.msh", check="modules/testlab/tests/poisson_test_ref_L-shape_3D.txt",
        kind="testlab", f=5.5, dirichlet=[("bot", 50.0), ("bc", 10.0)], penalty=1e30, eps=1e-4, min_value=1e-16),
    # modules/testlab/inputs/Test.sphere.3D.csr-gpu.arc
    "testlab_sphere_3d": dict(
        mesh="meshes/msh/sphere_cut.msh", check="modules/testlab/tests/poisson_test_ref_sphere_3D.txt",
        kind="testlab", f=5.5, dirichlet=[("horizontal", 0.5)], penalty=1e31, eps=1e-4, min_value=1e-16),
    # modules/poisson/inputs/circle.2D.arc (also run with matrix-format=AF-BSR, CMakeLists.txt:254-265)
    "poisson_circle_2d": dict(
        mesh="meshes/msh/circle_cut.msh", check="modules/poisson/check/poisson_test_ref_circle_2D.txt",
        kind="poisson", f=5.5, dirichlet=[("horizontal", 0.5)], penalty=1e30, eps=1e-4, min_value=0.0),
    # modules/poisson/inputs/sphere.3D.arc
    "poisson_sphere_3d": dict(
        mesh="meshes/msh/sphere_cut.msh", check="modules/poisson/check/poisson_test_ref_sphere_3D.txt",
        kind="poisson", f=5.5, dirichlet=[("horizontal", 0.5)], penalty=1e30, eps=1e-4, min_value=0.0),
    # modules/elasticity/inputs/bar.3D.Dirichlet.bodyForce.arc (f = "-1.0": x component only)
    "elasticity_bar_3d": dict(
        mesh="meshes/msh/bar_dynamic_3D.msh", check="modules/elasticity/check/bar.3D.Dirichlet.bodyForce.txt",
        kind="elasticity", E=21.0e5, nu=0.28, body_force=[-1.0, 0.0, 0.0],
        dirichlet3=[("surfaceleft", [0.0, 0.0, 0.0]), ("surfaceright", [None, 1.0, None])],
        penalty=1e30, eps=1e-3, min_value=1e-10),
}

def build_case(root: str, name: str, spec: dict) -> dict:
    """Mesh through the library's gmsh MSH 4.1 reader (node local ids in
    increasing gmsh tag order), check file as given."""
    d = meshio.read_msh(os.path.join(root, spec["mesh"]))
    coords, cells, tags_sorted, groups = d.mesh.coords, d.mesh.cells, d.node_tags, d.mesh.groups
    check = np.loadtxt(os.path.join(root, spec["check"]))
    out = dict(coords=coords.astype(np.float64), cells=cells, node_tags=tags_sorted.astype(np.int64),
               check_uid=check[:, 0].astype(np.int64), check_val=check[:, 1:].astype(np.float64))
    for g, ids in groups.items():
        out["group__" + g] = ids
    return out


def main(root: str) -> None:
    for name, spec in CASES.items():
        arrays = build_case(root, name, spec)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **arrays)
        print(f"{name}: nodes={arrays['coords'].shape[0]} cells={arrays['cells'].shape} "
              f"groups={[k[7:] for k in arrays if k.startswith('group__')]} -> {os.path.basename(path)}")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ARCANEFEM_REFERENCE")
    if not root:
        sys.exit("usage: make_fixtures.py <reference source tree>  (or set ARCANEFEM_REFERENCE)")
    main(root)
