"""Mesh input and solution output on the host.

* ``read_msh``: gmsh MSH 4.1 (binary little-endian with 8-byte sizes, or
  ASCII), the format of ArcaneFEM's meshes (``meshes/msh``).  The reader
  follows the public MSH 4.1 specification: ``$PhysicalNames``,
  ``$Entities``, ``$Nodes``, ``$Elements``; other sections are skipped.
  Node local ids follow increasing gmsh node tag (Arcane's numbering of a
  gmsh mesh, which the reference's check files use as node uids); cells are
  the highest-dimension elements (triangles, quadrangles, tetrahedra,
  hexahedra); each physical group of lower dimension gives a node group and,
  for faces (dimension cell_dim - 1), a face group with orientation flags
  for ``afem_rhs_boundary_faces``.
* ``write_msh``: binary MSH 4.1 of a ``meshgen.Mesh`` with its node groups
  (as point-element physical groups), so that synthetic meshes can be fed to
  other tools.
* ``write_vtu``: VTK XML unstructured grid (base64 inline binary) with point
  and cell data, for inspecting solutions in ParaView.  The reference writes
  VTKHDF / Ensight through Arcane; VTKHDF needs HDF5, which this image lacks.
"""
from __future__ import annotations

import base64
import struct
from dataclasses import dataclass, field

import numpy as np

from .meshgen import Mesh

# gmsh element type -> (nodes, dimension)
GMSH_TYPES = {15: (1, 0), 1: (2, 1), 2: (3, 2), 3: (4, 2), 4: (4, 3), 5: (8, 3)}
CELL_TYPES = {(2, 3): 2, (2, 4): 3, (3, 4): 4, (3, 8): 5}     # (dim, nodes per cell) -> gmsh type
VTK_TYPES = {2: 5, 3: 9, 4: 10, 5: 12}                         # gmsh type -> VTK cell type


@dataclass
class MshData:
    mesh: Mesh
    node_tags: np.ndarray                                      # gmsh tag of each local node
    faces: dict = field(default_factory=dict)                  # name -> (face nodes [nf][k], outward [nf])


class _Reader:
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


def _read_raw(path: str):
    r = _Reader(open(path, "rb").read())
    binary = True
    names, ent_phys, tags, xyz, elems = {}, {}, [], [], []
    while r.p < len(r.d):
        head = r.line()
        if head == "$MeshFormat":
            ver, ftype, dsize = r.line().split()
            if ver != "4.1" or dsize != "8":
                raise ValueError(f"{path}: MSH {ver} with {dsize}-byte sizes; only 4.1 with 8-byte sizes is read")
            binary = ftype == "1"
            if binary:
                one, = r.take("<i")
                if one != 1:
                    raise ValueError(f"{path}: big-endian binary MSH is not read")
                r.line()
            if r.line() != "$EndMeshFormat":
                raise ValueError(f"{path}: malformed $MeshFormat")
        elif head == "$PhysicalNames":
            for _ in range(int(r.line())):
                dim, tag, rest = r.line().split(" ", 2)
                names[(int(dim), int(tag))] = rest.strip().strip('"')
            r.line()
        elif head == "$Entities":
            if binary:
                counts = r.take("<4Q")
                for dim, cnt in enumerate(counts):
                    for _ in range(cnt):
                        tag, = r.take("<i")
                        r.take("<3d" if dim == 0 else "<6d")
                        nph, = r.take("<Q")
                        ent_phys[(dim, tag)] = list(r.take(f"<{nph}i"))
                        if dim > 0:
                            nb, = r.take("<Q")
                            r.take(f"<{nb}i")
                r.line()
            else:
                counts = [int(v) for v in r.line().split()]
                for dim, cnt in enumerate(counts):
                    for _ in range(cnt):
                        v = r.line().split()
                        tag = int(v[0])
                        k = 4 if dim == 0 else 7
                        nph = int(v[k])
                        ent_phys[(dim, tag)] = [int(x) for x in v[k + 1:k + 1 + nph]]
            if r.line() != "$EndEntities":
                raise ValueError(f"{path}: malformed $Entities")
        elif head == "$Nodes":
            if binary:
                nblk, _, _, _ = r.take("<4Q")
                for _ in range(nblk):
                    _, _, param = r.take("<3i")
                    n, = r.take("<Q")
                    if param:
                        raise ValueError(f"{path}: parametric node blocks are not read")
                    tags.append(r.arr("<u8", n).astype(np.int64))
                    xyz.append(r.arr("<f8", n * 3).reshape(n, 3))
                r.line()
            else:
                nblk = int(r.line().split()[0])
                for _ in range(nblk):
                    v = r.line().split()
                    n = int(v[3])
                    if int(v[2]):
                        raise ValueError(f"{path}: parametric node blocks are not read")
                    tags.append(np.array([int(r.line()) for _ in range(n)], np.int64))
                    xyz.append(np.array([[float(c) for c in r.line().split()[:3]] for _ in range(n)]).reshape(n, 3))
            if r.line() != "$EndNodes":
                raise ValueError(f"{path}: malformed $Nodes")
        elif head == "$Elements":
            if binary:
                nblk, _, _, _ = r.take("<4Q")
                for _ in range(nblk):
                    edim, etag, etype = r.take("<3i")
                    n, = r.take("<Q")
                    if etype not in GMSH_TYPES:
                        raise ValueError(f"{path}: gmsh element type {etype} is not read")
                    k = GMSH_TYPES[etype][0]
                    data = r.arr("<u8", n * (k + 1)).reshape(n, k + 1).astype(np.int64)
                    elems.append((edim, etag, etype, data[:, 1:]))
                r.line()
            else:
                nblk = int(r.line().split()[0])
                for _ in range(nblk):
                    edim, etag, etype, n = (int(v) for v in r.line().split())
                    if etype not in GMSH_TYPES:
                        raise ValueError(f"{path}: gmsh element type {etype} is not read")
                    data = np.array([[int(c) for c in r.line().split()] for _ in range(n)], np.int64)
                    elems.append((edim, etag, etype, data[:, 1:].reshape(n, -1)))
            if r.line() != "$EndElements":
                raise ValueError(f"{path}: malformed $Elements")
        elif head.startswith("$"):
            end = ("$End" + head[1:]).encode()
            r.p = r.d.index(end, r.p)
            r.line()
    if not tags or not elems:
        raise ValueError(f"{path}: no nodes or elements")
    return names, ent_phys, np.concatenate(tags), np.concatenate(xyz), elems


def face_outward(mesh: Mesh, faces: np.ndarray) -> np.ndarray:
    """Orientation flag of boundary faces of a simplex mesh: 1 when the node
    order gives the outward normal (edge (dy, -dx), triangle (n1-n0) x (n2-n0)),
    0 otherwise (Arcane's isSubDomainBoundaryOutside).  A face that bounds no
    cell keeps 1."""
    faces = np.asarray(faces, np.int64)
    c = np.asarray(mesh.cells, np.int64)
    k = c.shape[1]
    cf, opp = [], []
    for skip in range(k):
        cf.append(np.delete(c, skip, axis=1))
        opp.append(c[:, skip])
    cf = np.sort(np.concatenate(cf), axis=1)
    opp = np.concatenate(opp)
    base = int(max(c.max(), faces.max())) + 1
    def code(a):
        v = np.zeros(a.shape[0], np.int64)
        for col in range(a.shape[1]):
            v = v * base + a[:, col]
        return v
    ck = code(cf)
    order = np.argsort(ck)
    fk = code(np.sort(faces, axis=1))
    pos = np.clip(np.searchsorted(ck[order], fk), 0, ck.size - 1)
    found = ck[order][pos] == fk
    o = opp[order][pos]
    X = mesh.coords
    if mesh.dim == 2:
        d = X[faces[:, 1], :2] - X[faces[:, 0], :2]
        nrm = np.stack([d[:, 1], -d[:, 0]], 1)
        away = X[o, :2] - X[faces[:, 0], :2]
    else:
        nrm = np.cross(X[faces[:, 1]] - X[faces[:, 0]], X[faces[:, 2]] - X[faces[:, 0]])
        away = X[o] - X[faces[:, 0]]
    out = (np.einsum("ij,ij->i", nrm, away) < 0).astype(np.uint8)
    out[~found] = 1
    return out


def read_msh(path: str) -> MshData:
    names, ent_phys, tags, xyz, elems = _read_raw(path)
    order = np.argsort(tags, kind="stable")
    tags_sorted = tags[order]
    lut = np.full(int(tags_sorted.max()) + 1, -1, np.int64)
    lut[tags_sorted] = np.arange(tags_sorted.size)
    cell_dim = max(GMSH_TYPES[e[2]][1] for e in elems)
    cell_blocks = [e for e in elems if GMSH_TYPES[e[2]][1] == cell_dim]
    if len({e[2] for e in cell_blocks}) != 1:
        raise ValueError(f"{path}: mixed cell types are not supported")
    cells = lut[np.concatenate([e[3] for e in cell_blocks])].astype(np.int32)
    groups, face_nodes = {}, {}
    for (pdim, ptag), pname in names.items():
        sel, fsel = [], []
        for edim, etag, etype, enodes in elems:
            if GMSH_TYPES[etype][1] == pdim and ptag in ent_phys.get((edim, etag), []):
                sel.append(enodes.ravel())
                if pdim == cell_dim - 1:
                    fsel.append(lut[enodes])
        if sel:
            groups[pname] = np.unique(lut[np.concatenate(sel)]).astype(np.int32)
        if fsel:
            face_nodes[pname] = np.concatenate(fsel).astype(np.int32)
    mesh = Mesh(cell_dim, xyz[order].astype(np.float64), cells, groups)
    faces = {}
    simplex = cells.shape[1] == cell_dim + 1
    for name, f in face_nodes.items():
        faces[name] = (f, face_outward(mesh, f) if simplex else np.ones(len(f), np.uint8))
    return MshData(mesh, tags_sorted.astype(np.int64), faces)


def write_msh(path: str, mesh: Mesh) -> None:
    """Binary MSH 4.1: one volume entity holding the cells, one point entity
    per node group (physical name = group name, point elements)."""
    cells = np.asarray(mesh.cells, np.int64)
    etype = CELL_TYPES[(mesh.dim, cells.shape[1])]
    names = sorted(mesh.groups)
    out = bytearray()
    out += b"$MeshFormat\n4.1 1 8\n" + struct.pack("<i", 1) + b"\n$EndMeshFormat\n"
    out += f"$PhysicalNames\n{len(names) + 1}\n".encode()
    out += f'{mesh.dim} 1 "cells"\n'.encode()
    for i, g in enumerate(names):
        out += f'0 {i + 2} "{g}"\n'.encode()
    out += b"$EndPhysicalNames\n$Entities\n"
    counts = [len(names), 0, 0, 0]
    counts[mesh.dim] += 1
    out += struct.pack("<4Q", *counts)
    for i, g in enumerate(names):          # point entities 1..G, physical i+2
        out += struct.pack("<i3dQi", i + 1, 0.0, 0.0, 0.0, 1, i + 2)
    lo, hi = mesh.coords.min(0), mesh.coords.max(0)
    out += struct.pack("<i6dQiQ", 1, *lo, *hi, 1, 1, 0)
    out += b"\n$EndEntities\n$Nodes\n"
    n = mesh.nb_node
    out += struct.pack("<4Q", 1, n, 1, n)
    out += struct.pack("<3iQ", mesh.dim, 1, 0, n)
    out += np.arange(1, n + 1, dtype="<u8").tobytes() + np.asarray(mesh.coords, "<f8").tobytes()
    out += b"\n$EndNodes\n$Elements\n"
    nel = cells.shape[0] + sum(len(mesh.groups[g]) for g in names)
    out += struct.pack("<4Q", 1 + len(names), nel, 1, nel)
    out += struct.pack("<3iQ", mesh.dim, 1, etype, cells.shape[0])
    blk = np.concatenate([np.arange(1, cells.shape[0] + 1)[:, None], cells + 1], axis=1).astype("<u8")
    out += blk.tobytes()
    next_tag = cells.shape[0] + 1
    for i, g in enumerate(names):
        ids = np.asarray(mesh.groups[g], np.int64)
        out += struct.pack("<3iQ", 0, i + 1, 15, ids.size)
        blk = np.stack([np.arange(next_tag, next_tag + ids.size), ids + 1], axis=1).astype("<u8")
        out += blk.tobytes()
        next_tag += ids.size
    out += b"\n$EndElements\n"
    with open(path, "wb") as f:
        f.write(bytes(out))


def _b64(a: np.ndarray) -> str:
    raw = np.ascontiguousarray(a).tobytes()
    return base64.b64encode(struct.pack("<Q", len(raw)) + raw).decode()


def write_vtu(path: str, mesh: Mesh, point_data: dict | None = None, cell_data: dict | None = None) -> None:
    """VTK XML unstructured grid, little-endian, UInt64 headers, base64 binary."""
    cells = np.asarray(mesh.cells, np.int64)
    etype = CELL_TYPES[(mesh.dim, cells.shape[1])]
    n, c, k = mesh.nb_node, cells.shape[0], cells.shape[1]

    def data_array(name, a):
        a = np.asarray(a)
        ncomp = 1 if a.ndim == 1 else a.shape[1]
        t = {np.dtype("float64"): "Float64", np.dtype("float32"): "Float32", np.dtype("int32"): "Int32",
             np.dtype("int64"): "Int64", np.dtype("uint8"): "UInt8"}[a.dtype]
        return (f'<DataArray type="{t}" Name="{name}" NumberOfComponents="{ncomp}" format="binary">'
                f"{_b64(a.astype(a.dtype.newbyteorder('<')))}</DataArray>\n")

    s = ['<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="1.0" byte_order="LittleEndian" '
         'header_type="UInt64">\n<UnstructuredGrid>\n', f'<Piece NumberOfPoints="{n}" NumberOfCells="{c}">\n']
    s.append("<PointData>\n")
    for name, a in (point_data or {}).items():
        s.append(data_array(name, a))
    s.append("</PointData>\n<CellData>\n")
    for name, a in (cell_data or {}).items():
        s.append(data_array(name, a))
    s.append("</CellData>\n<Points>\n")
    s.append(data_array("Points", np.asarray(mesh.coords, np.float64)))
    s.append("</Points>\n<Cells>\n")
    s.append(data_array("connectivity", cells.ravel()))
    s.append(data_array("offsets", np.arange(k, k * c + 1, k, dtype=np.int64)))
    s.append(data_array("types", np.full(c, VTK_TYPES[etype], np.uint8)))
    s.append("</Cells>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n")
    with open(path, "w") as f:
        f.write("".join(s))
