"""Seeded synthetic P1 meshes: jittered structured triangles and tetrahedra.

These stand in for the gmsh meshes ArcaneFEM reads (the benchmark meshes of
modules/testlab/benchmarking/run-benchmark.sh are not shipped).  Layout is
the one the C ABI takes: ``coords`` float64 [nb_node, 3] (z = 0 in 2D) and
``cells`` int32 [nb_cell, 3|4].

* Unit square, n x n quads, each split along the SW-NE diagonal into two
  counter-clockwise triangles.  Node id = i + j (n+1).
* Unit cube, n^3 hexahedra, each split into the 6 Kuhn tetrahedra that share
  the main diagonal (a conforming split), ordered to have positive volume.
  Node id = i + j (n+1) + k (n+1)^2.
* Interior nodes are moved by U[-a h, a h] per component (numpy PCG64 from
  the seed); boundary nodes stay on the boundary.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from itertools import permutations

import numpy as np


@dataclass
class Mesh:
    dim: int
    coords: np.ndarray            # float64 [N, 3]
    cells: np.ndarray             # int32 [C, npc]
    groups: dict = field(default_factory=dict)   # name -> int32 node ids

    @property
    def nb_node(self) -> int:
        return int(self.coords.shape[0])

    @property
    def nb_cell(self) -> int:
        return int(self.cells.shape[0])

    @property
    def npc(self) -> int:
        return int(self.cells.shape[1])


def _jitter(coords: np.ndarray, interior: np.ndarray, amp: float, rng: np.random.Generator, dim: int) -> None:
    nb = int(interior.sum())
    delta = rng.uniform(-amp, amp, size=(nb, dim))
    coords[interior, :dim] += delta


def unit_square_tri(n: int, jitter: float = 0.2, seed: int = 0) -> Mesh:
    h = 1.0 / n
    m = n + 1
    ii, jj = np.meshgrid(np.arange(m), np.arange(m), indexing="xy")      # jj rows, ii cols
    coords = np.zeros((m * m, 3))
    coords[:, 0] = (ii.ravel() * h)
    coords[:, 1] = (jj.ravel() * h)
    ids = np.arange(m * m).reshape(m, m)     # ids[j, i] = i + j m
    interior = np.zeros((m, m), bool)
    interior[1:-1, 1:-1] = True
    interior = interior.ravel()
    if jitter > 0:
        _jitter(coords, interior, jitter * h, np.random.default_rng(seed), 2)
    sw = ids[:-1, :-1].ravel()
    se = ids[:-1, 1:].ravel()
    ne = ids[1:, 1:].ravel()
    nw = ids[1:, :-1].ravel()
    cells = np.empty((n * n * 2, 3), np.int32)
    cells[0::2] = np.stack([sw, se, ne], 1)
    cells[1::2] = np.stack([sw, ne, nw], 1)
    x, y = coords[:, 0], coords[:, 1]
    eps = 1e-12
    groups = {
        "boundary": np.flatnonzero(~interior).astype(np.int32),
        "left": np.flatnonzero(np.abs(x) < eps).astype(np.int32),
        "right": np.flatnonzero(np.abs(x - 1) < eps).astype(np.int32),
        "bottom": np.flatnonzero(np.abs(y) < eps).astype(np.int32),
        "top": np.flatnonzero(np.abs(y - 1) < eps).astype(np.int32),
    }
    return Mesh(2, coords, cells, groups)


def _kuhn_tets():
    """The 6 Kuhn tetrahedra of the unit cube as local hex-corner indices
    (corner index = dx + 2 dy + 4 dz), each ordered for positive volume."""
    tets = []
    for perm in permutations(range(3)):
        path = [0]
        cur = 0
        for a in perm:
            cur |= 1 << a
            path.append(cur)
        # parity of the permutation decides the orientation
        inv = sum(1 for i in range(3) for j in range(i + 1, 3) if perm[i] > perm[j])
        if inv % 2 == 1:
            path[1], path[2] = path[2], path[1]
        tets.append(path)
    return np.array(tets, np.int64)


def unit_cube_tet(n: int, jitter: float = 0.15, seed: int = 0) -> Mesh:
    h = 1.0 / n
    m = n + 1
    kk, jj, ii = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    coords = np.zeros((m ** 3, 3))
    coords[:, 0] = ii.ravel() * h
    coords[:, 1] = jj.ravel() * h
    coords[:, 2] = kk.ravel() * h
    interior = np.zeros((m, m, m), bool)
    interior[1:-1, 1:-1, 1:-1] = True
    interior = interior.ravel()
    if jitter > 0:
        _jitter(coords, interior, jitter * h, np.random.default_rng(seed), 3)
    # hex origin ids, hex index = i + j n + k n^2
    k0, j0, i0 = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    base = (i0 + j0 * m + k0 * m * m).ravel().astype(np.int64)
    corner = np.array([dx + dy * m + dz * m * m for dz in (0, 1) for dy in (0, 1) for dx in (0, 1)], np.int64)
    kt = _kuhn_tets()
    cells = (base[:, None, None] + corner[kt][None, :, :]).reshape(-1, 4).astype(np.int32)
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    eps = 1e-12
    groups = {
        "boundary": np.flatnonzero(~interior).astype(np.int32),
        "xmin": np.flatnonzero(np.abs(x) < eps).astype(np.int32),
        "xmax": np.flatnonzero(np.abs(x - 1) < eps).astype(np.int32),
        "zmin": np.flatnonzero(np.abs(z) < eps).astype(np.int32),
    }
    groups["x_faces"] = np.union1d(groups["xmin"], groups["xmax"]).astype(np.int32)
    return Mesh(3, coords, cells, groups)


def signed_measures(mesh: Mesh) -> np.ndarray:
    """Signed area (2D) or 6x signed volume (3D) of every cell (host check)."""
    c = mesh.coords
    e = mesh.cells
    if mesh.dim == 2:
        a = c[e[:, 1]] - c[e[:, 0]]
        b = c[e[:, 2]] - c[e[:, 0]]
        return 0.5 * (a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0])
    v0 = c[e[:, 1]] - c[e[:, 0]]
    v1 = c[e[:, 2]] - c[e[:, 0]]
    v2 = c[e[:, 3]] - c[e[:, 0]]
    return np.einsum("ij,ij->i", v0, np.cross(v1, v2))


def nnz_formula(mesh: Mesh) -> int:
    """nb_node + 2 nb_edge (NodeWiseCsrBiliAssembly.cc:121, BSRFormat.cc:278-283)."""
    e = mesh.cells.astype(np.int64)
    npc = mesh.npc
    pairs = []
    for a in range(npc):
        for b in range(a + 1, npc):
            lo = np.minimum(e[:, a], e[:, b])
            hi = np.maximum(e[:, a], e[:, b])
            pairs.append(lo << 32 | hi)
    nb_edge = np.unique(np.concatenate(pairs)).size
    return mesh.nb_node + 2 * nb_edge


def boundary_faces(mesh: Mesh, seed: int = 0):
    """Boundary faces of a P1 mesh (edges of triangles, triangles of tets),
    each in a random node order, with its orientation flag: 1 when the order
    gives the outward normal (edge: (dy, -dx); triangle: (n1-n0) x (n2-n0)),
    0 when the first two nodes must be swapped for it (Arcane's
    isSubDomainBoundaryOutside).  Faces come sorted by their node set."""
    rng = np.random.default_rng(seed)
    c = mesh.cells
    if mesh.dim == 2:
        loc = [(0, 1, 2), (1, 2, 0), (2, 0, 1)]   # edge (a, b), opposite vertex
    else:
        loc = [(1, 2, 3, 0), (0, 2, 3, 1), (0, 1, 3, 2), (0, 1, 2, 3)]
    faces, opp = [], []
    for t in loc:
        faces.append(c[:, list(t[:-1])])
        opp.append(c[:, t[-1]])
    faces = np.concatenate(faces)
    opp = np.concatenate(opp)
    key = np.sort(faces, axis=1)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    bnd = cnt[inv.ravel()] == 1
    f, o = faces[bnd], opp[bnd]
    order = np.lexsort(np.sort(f, axis=1).T[::-1])
    f, o = f[order], o[order]
    # random node order per face
    perm = np.array([rng.permutation(f.shape[1]) for _ in range(f.shape[0])]) if f.shape[0] else np.zeros((0, f.shape[1]), int)
    f = np.take_along_axis(f, perm, axis=1).astype(np.int32)
    X = mesh.coords
    if mesh.dim == 2:
        d = X[f[:, 1], :2] - X[f[:, 0], :2]
        nrm = np.stack([d[:, 1], -d[:, 0]], 1)
        away = X[o, :2] - X[f[:, 0], :2]
    else:
        nrm = np.cross(X[f[:, 1]] - X[f[:, 0]], X[f[:, 2]] - X[f[:, 0]])
        away = X[o] - X[f[:, 0]]
    outward = (np.einsum("ij,ij->i", nrm, away) < 0).astype(np.uint8)
    return f, outward


def unit_square_quad(n: int, jitter: float = 0.2, seed: int = 0) -> Mesh:
    """n x n bilinear quadrilaterals of the unit square, counter-clockwise
    (the Quad4 reference order), node id = i + j (n+1), interior nodes jittered."""
    tri = unit_square_tri(n, jitter=jitter, seed=seed)
    m = n + 1
    ids = np.arange(m * m).reshape(m, m)
    q = np.stack([ids[:-1, :-1], ids[:-1, 1:], ids[1:, 1:], ids[1:, :-1]], axis=-1).reshape(-1, 4)
    return Mesh(2, tri.coords, q.astype(np.int32), dict(tri.groups))


def unit_cube_hex(n: int, jitter: float = 0.15, seed: int = 0) -> Mesh:
    """n^3 trilinear hexahedra of the unit cube in the Hexa8 reference order
    (bottom face counter-clockwise, then the top face), node id =
    i + j (n+1) + k (n+1)^2, interior nodes jittered."""
    tet = unit_cube_tet(n, jitter=jitter, seed=seed)
    m = n + 1
    ids = np.arange(m ** 3).reshape(m, m, m)   # [k][j][i]
    b = [ids[:-1, :-1, :-1], ids[:-1, :-1, 1:], ids[:-1, 1:, 1:], ids[:-1, 1:, :-1]]
    t = [ids[1:, :-1, :-1], ids[1:, :-1, 1:], ids[1:, 1:, 1:], ids[1:, 1:, :-1]]
    h = np.stack(b + t, axis=-1).reshape(-1, 8)
    return Mesh(3, tet.coords, h.astype(np.int32), dict(tet.groups))
