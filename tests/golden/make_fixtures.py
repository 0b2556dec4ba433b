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
import struct
import sys

import numpy as np

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

ELEM_NODES = {1: 2, 2: 3, 3: 4, 4: 4, 5: 8, 15: 1}


class Reader:
    def __init__(self, data: bytes):
        self.d = data
        self.p = 0

    def line(self) -> str:
        e = self.d.index(b"\n", self.p)
        s = self.d[self.p:e].decode()
        self.p = e + 1
        return s.strip()

    def take(self, fmt: str):
        n = struct.calcsize(fmt)
        v = struct.unpack_from(fmt, self.d, self.p)
        self.p += n
        return v

    def arr(self, dtype, count):
        a = np.frombuffer(self.d, dtype=dtype, count=count, offset=self.p)
        self.p += a.nbytes
        return a


def read_msh41(path: str):
    """Minimal reader of binary gmsh 4.1 (public format specification):
    physical names, entities, nodes and elements."""
    r = Reader(open(path, "rb").read())
    names = {}
    ent_phys = {}
    nodes_tag = []
    nodes_xyz = []
    elems = []   # (dim, entity_tag, type, tags[n], node_tags[n, k])
    while r.p < len(r.d):
        head = r.line()
        if head == "$MeshFormat":
            ver, ftype, dsize = r.line().split()
            assert ver == "4.1" and ftype == "1" and dsize == "8", (ver, ftype, dsize)
            one, = r.take("<i")
            assert one == 1
            r.line()
            assert r.line() == "$EndMeshFormat"
        elif head == "$PhysicalNames":
            n = int(r.line())
            for _ in range(n):
                s = r.line()
                dim, tag, rest = s.split(" ", 2)
                names[(int(dim), int(tag))] = rest.strip().strip('"')
            assert r.line() == "$EndPhysicalNames"
        elif head == "$Entities":
            npt, ncu, nsu, nvo = r.take("<4Q")
            for _ in range(npt):
                tag, = r.take("<i")
                r.take("<3d")
                nph, = r.take("<Q")
                ent_phys[(0, tag)] = list(r.take(f"<{nph}i"))
            for dim, cnt in ((1, ncu), (2, nsu), (3, nvo)):
                for _ in range(cnt):
                    tag, = r.take("<i")
                    r.take("<6d")
                    nph, = r.take("<Q")
                    ent_phys[(dim, tag)] = list(r.take(f"<{nph}i"))
                    nb, = r.take("<Q")
                    r.take(f"<{nb}i")
            r.line()
            assert r.line() == "$EndEntities"
        elif head == "$Nodes":
            nblk, nnod, _, _ = r.take("<4Q")
            for _ in range(nblk):
                edim, etag, param = r.take("<3i")
                n, = r.take("<Q")
                tags = r.arr("<u8", n).astype(np.int64)
                xyz = r.arr("<f8", n * 3).reshape(n, 3)
                assert param == 0
                nodes_tag.append(tags)
                nodes_xyz.append(xyz)
            r.line()
            assert r.line() == "$EndNodes"
        elif head == "$Elements":
            nblk, nel, _, _ = r.take("<4Q")
            for _ in range(nblk):
                edim, etag, etype = r.take("<3i")
                n, = r.take("<Q")
                k = ELEM_NODES[etype]
                data = r.arr("<u8", n * (k + 1)).reshape(n, k + 1).astype(np.int64)
                elems.append((edim, etag, etype, data[:, 0], data[:, 1:]))
            r.line()
            assert r.line() == "$EndElements"
        elif head.startswith("$"):
            end = "$End" + head[1:]
            idx = r.d.index(end.encode(), r.p)
            r.p = idx
            r.line()
        else:
            continue
    tags = np.concatenate(nodes_tag)
    xyz = np.concatenate(nodes_xyz)
    return names, ent_phys, tags, xyz, elems


def build_case(root: str, name: str, spec: dict) -> dict:
    names, ent_phys, tags, xyz, elems = read_msh41(os.path.join(root, spec["mesh"]))
    cell_dim = max(e[0] for e in elems)
    order = np.argsort(tags)
    tags_sorted = tags[order]
    # node local ids follow increasing gmsh node tag
    coords = xyz[order]
    tag_to_lid = {int(t): i for i, t in enumerate(tags_sorted)}
    cells = [e[4] for e in elems if e[0] == cell_dim]
    cells = np.concatenate(cells)
    cells = np.vectorize(tag_to_lid.__getitem__)(cells).astype(np.int32)
    groups = {}
    for (pdim, ptag), pname in names.items():
        sel = []
        for edim, etag, etype, etags, enodes in elems:
            if edim == pdim and ptag in ent_phys.get((edim, etag), []):
                sel.append(enodes.ravel())
        if sel:
            ids = np.unique(np.concatenate(sel))
            groups[pname] = np.array([tag_to_lid[int(t)] for t in ids], np.int32)
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
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
