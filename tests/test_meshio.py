"""Mesh I/O: gmsh MSH 4.1 round trips (binary writer -> reader), the
reference's own meshes against the committed fixtures when the reference tree
is present, face groups with orientation flags, and the VTU writer."""
import base64
import os
import struct
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from arcanefem_gb300 import meshgen, meshio

# the reference source tree, when a checkout is at hand: ARCANEFEM_REFERENCE=<tree>
REF = os.path.join(os.environ.get("ARCANEFEM_REFERENCE", ""), "meshes", "msh")
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.parametrize("make", [lambda: meshgen.unit_square_tri(6, seed=1), lambda: meshgen.unit_cube_tet(3, seed=2),
                                  lambda: meshgen.unit_square_quad(5, seed=3), lambda: meshgen.unit_cube_hex(3, seed=4)])
def test_msh_round_trip(tmp_path, make):
    m = make()
    path = str(tmp_path / "m.msh")
    meshio.write_msh(path, m)
    d = meshio.read_msh(path)
    assert d.mesh.dim == m.dim
    assert np.array_equal(d.mesh.coords, m.coords) and np.array_equal(d.mesh.cells, m.cells)
    assert set(d.mesh.groups) >= set(m.groups)
    for g, ids in m.groups.items():
        assert np.array_equal(d.mesh.groups[g], np.unique(ids))
    assert np.array_equal(d.node_tags, np.arange(1, m.nb_node + 1))


@pytest.mark.skipif(not os.environ.get("ARCANEFEM_REFERENCE") or not os.path.isdir(REF),
                    reason="ARCANEFEM_REFERENCE does not name a reference tree with meshes/msh")
@pytest.mark.parametrize("name,fixture", [("L-shape.msh", "testlab_lshape_2d.npz"),
                                          ("circle_cut.msh", "poisson_circle_2d.npz"),
                                          ("bar_dynamic_3D.msh", "elasticity_bar_3d.npz")])
def test_reads_the_reference_meshes(name, fixture):
    fx = os.path.join(HERE, "golden", fixture)
    if not os.path.exists(fx):
        pytest.skip("fixture missing")
    d = meshio.read_msh(os.path.join(REF, name))
    g = np.load(fx)
    assert np.array_equal(d.mesh.coords, g["coords"]) and np.array_equal(d.mesh.cells, g["cells"])
    assert np.array_equal(d.node_tags, g["node_tags"])
    for k in g.files:
        if k.startswith("group__"):
            assert np.array_equal(d.mesh.groups[k[7:]], g[k]), k


def test_face_groups_are_oriented(tmp_path):
    m = meshgen.unit_cube_tet(3, seed=5)
    f, out = meshgen.boundary_faces(m, seed=6)
    assert np.array_equal(meshio.face_outward(m, f), out)
    m2 = meshgen.unit_square_tri(5, seed=7)
    f2, out2 = meshgen.boundary_faces(m2, seed=8)
    assert np.array_equal(meshio.face_outward(m2, f2), out2)


def _decode(el):
    raw = base64.b64decode(el.text)
    n, = struct.unpack_from("<Q", raw)
    t = {"Float64": "<f8", "Int64": "<i8", "UInt8": "u1", "Int32": "<i4", "Float32": "<f4"}[el.get("type")]
    return np.frombuffer(raw[8:8 + n], dtype=t)


def test_vtu_writer(tmp_path):
    m = meshgen.unit_cube_tet(2, seed=1)
    u = np.linspace(0, 1, m.nb_node)
    path = str(tmp_path / "u.vtu")
    meshio.write_vtu(path, m, point_data={"u": u}, cell_data={"k": np.ones(m.nb_cell)})
    root = ET.parse(path).getroot()
    piece = root.find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfPoints")) == m.nb_node and int(piece.get("NumberOfCells")) == m.nb_cell
    arrays = {e.get("Name"): e for e in root.iter("DataArray")}
    assert np.array_equal(_decode(arrays["u"]), u)
    assert np.array_equal(_decode(arrays["connectivity"]).reshape(-1, 4), m.cells)
    assert np.array_equal(_decode(arrays["Points"]).reshape(-1, 3), m.coords)
    assert set(_decode(arrays["types"]).tolist()) == {10}
