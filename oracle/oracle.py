"""ctypes binding of the CPU oracle (liboracle_afem.so).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path.  Imported by tests/,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs, never by the
``arcanefem_gb300`` package.  Each wrapper mirrors a function of
``afem_oracle.h``, which cites the ArcaneFEM source it restates.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle_afem.so")
_lib = None

POISSON_TRI3, POISSON_TET4, ELASTICITY_TET4, TESTLAB_TRI3, TESTLAB_TET4 = 0, 1, 2, 3, 4
POISSON_QUAD4, POISSON_HEXA8 = 5, 6
ELIM_NONE, ELIM_ROW, ELIM_ROW_COLUMN = 0, 1, 2


def build() -> str:
    """Compile liboracle_afem.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = C.CDLL(_LIB_PATH)
        _declare(_lib)
    return _lib


_P = C.c_void_p


def _declare(L):
    L.afo_node_cell.argtypes = [C.c_int, C.c_int, C.c_int, _P, _P, _P, _P]
    L.afo_node_cell.restype = C.c_int
    L.afo_sparsity.argtypes = [C.c_int, C.c_int, C.c_int, _P, C.c_int, _P, _P, C.c_int64]
    L.afo_sparsity.restype = C.c_int64
    for name in ("afo_elem_vec_poisson_tri3", "afo_elem_vec_poisson_tet4", "afo_elem_vec_testlab_tri3",
                 "afo_elem_vec_testlab_tet4"):
        getattr(L, name).argtypes = [_P, _P, C.c_int, _P]
        getattr(L, name).restype = None
    L.afo_elem_vec_elasticity_tet4.argtypes = [_P, _P, C.c_double, C.c_double, C.c_int, _P]
    L.afo_elem_vec_elasticity_tet4.restype = None
    L.afo_assemble_nodewise.argtypes = [C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, _P, C.c_int,
                                        C.c_double, C.c_double, _P, _P, C.c_int]
    L.afo_assemble_nodewise.restype = C.c_int
    L.afo_rhs_constant_source.argtypes = [C.c_int, C.c_int, _P, _P, C.c_int, _P, _P, C.c_double, C.c_int, _P]
    L.afo_rhs_constant_source.restype = None
    L.afo_rhs_body_force_tet4.argtypes = [C.c_int, _P, _P, _P, _P]
    L.afo_rhs_body_force_tet4.restype = None
    L.afo_rhs_boundary_faces.argtypes = [C.c_int, C.c_int, _P, _P, _P, C.c_int, _P, C.c_int, _P]
    L.afo_rhs_boundary_faces.restype = None
    L.afo_rhs_constant_source_q1.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P, C.c_double, C.c_int, _P]
    L.afo_rhs_constant_source_q1.restype = None
    L.afo_dirichlet_penalty.argtypes = [C.c_int, _P, C.c_int, C.c_int, C.c_double, C.c_double, _P, _P, _P]
    L.afo_dirichlet_penalty.restype = None
    L.afo_dirichlet_elimination.argtypes = [C.c_int, _P, C.c_int, C.c_int, C.c_double, C.c_uint8, _P, _P]
    L.afo_dirichlet_elimination.restype = None
    L.afo_apply_matrix_transformation.argtypes = [C.c_int, _P, _P, _P, _P, _P, _P, _P, _P, _P]
    L.afo_apply_matrix_transformation.restype = None
    L.afo_apply_rhs_transformation.argtypes = [C.c_int, _P, _P, _P, _P, _P, _P, _P]
    L.afo_apply_rhs_transformation.restype = None
    L.afo_spmv.argtypes = [C.c_int, _P, _P, _P, _P, _P]
    L.afo_spmv.restype = None
    L.afo_pcg_jacobi.argtypes = [C.c_int, _P, _P, _P, _P, _P, C.c_double, C.c_int, _P, _P, C.c_int]
    L.afo_pcg_jacobi.restype = C.c_int
    L.afo_assemble_dok.argtypes = [C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P, C.c_int64]
    L.afo_assemble_dok.restype = C.c_int64
    L.afo_sparsity_nodewise.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P, _P, C.c_int64, C.c_int]
    L.afo_sparsity_nodewise.restype = C.c_int64
    L.afo_wtime.argtypes = []
    L.afo_wtime.restype = C.c_double
    L.afo_max_threads.argtypes = []
    L.afo_max_threads.restype = C.c_int


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def max_threads() -> int:
    return int(lib().afo_max_threads())


def node_cell(nb_node, cell_nodes):
    cell_nodes = _c(cell_nodes, np.int32)
    nb_cell, npc = cell_nodes.shape
    ptr = np.zeros(nb_node + 1, np.int32)
    cells = np.zeros(nb_cell * npc, np.int32)
    local = np.zeros(nb_cell * npc, np.uint8)
    rc = lib().afo_node_cell(nb_node, nb_cell, npc, _p(cell_nodes), _p(ptr), _p(cells), _p(local))
    if rc != 0:
        raise ValueError("bad node id in cell connectivity")
    return ptr, cells, local


def sparsity(nb_node, cell_nodes, self_last=False):
    cell_nodes = _c(cell_nodes, np.int32)
    nb_cell, npc = cell_nodes.shape
    row_ptr = np.zeros(nb_node + 1, np.int32)
    cap = nb_node + nb_cell * npc * (npc - 1)
    cols = np.zeros(cap, np.int32)
    nnz = lib().afo_sparsity(nb_node, nb_cell, npc, _p(cell_nodes), int(self_last), _p(row_ptr), _p(cols), cap)
    if nnz < 0:
        raise RuntimeError("sparsity capacity too small")
    return row_ptr, cols[:nnz].copy()


def elem_vec(kind, coords, cell, local, lam=0.0, mu=0.0):
    coords = _c(coords, np.float64)
    cn = _c(cell, np.int32)
    L = lib()
    if kind == ELASTICITY_TET4:
        out = np.zeros(36)
        L.afo_elem_vec_elasticity_tet4(_p(coords), _p(cn), lam, mu, local, _p(out))
        return out.reshape(3, 12)
    fn = {POISSON_TRI3: L.afo_elem_vec_poisson_tri3, POISSON_TET4: L.afo_elem_vec_poisson_tet4,
          TESTLAB_TRI3: L.afo_elem_vec_testlab_tri3, TESTLAB_TET4: L.afo_elem_vec_testlab_tet4}[kind]
    out = np.zeros(4)
    fn(_p(coords), _p(cn), local, _p(out))
    return out[: cn.shape[0]]


def assemble(kind, coords, cell_nodes, nc_ptr, nc_cell, row_ptr, cols, per_block_layout=False, lam=0.0, mu=0.0,
             cell_coeff=None, nb_threads=1):
    coords = _c(coords, np.float64)
    cell_nodes = _c(cell_nodes, np.int32)
    b = 3 if kind == ELASTICITY_TET4 else 1
    nb_node = coords.shape[0]
    values = np.zeros(int(row_ptr[-1]) * b * b, np.float64)
    cc = None if cell_coeff is None else _c(cell_coeff, np.float64)
    rc = lib().afo_assemble_nodewise(kind, nb_node, cell_nodes.shape[0], _p(coords), _p(cell_nodes),
                                     _p(_c(nc_ptr, np.int32)), _p(_c(nc_cell, np.int32)), _p(_c(row_ptr, np.int32)),
                                     _p(_c(cols, np.int32)), int(per_block_layout), lam, mu, _p(cc), _p(values),
                                     int(nb_threads))
    if rc != 0:
        raise RuntimeError("column not found in row during assembly")
    return values


def rhs_constant_source(dim, coords, cell_nodes, nc_ptr, nc_cell, qdot, nb_dof=1):
    coords = _c(coords, np.float64)
    cell_nodes = _c(cell_nodes, np.int32)
    rhs = np.zeros(coords.shape[0] * nb_dof)
    lib().afo_rhs_constant_source(dim, coords.shape[0], _p(coords), _p(cell_nodes), cell_nodes.shape[1],
                                  _p(_c(nc_ptr, np.int32)), _p(_c(nc_cell, np.int32)), qdot, nb_dof, _p(rhs))
    return rhs


def rhs_body_force_tet4(coords, cell_nodes, f, rhs=None):
    coords = _c(coords, np.float64)
    cell_nodes = _c(cell_nodes, np.int32)
    if rhs is None:
        rhs = np.zeros(coords.shape[0] * 3)
    fv = _c(f, np.float64)
    lib().afo_rhs_body_force_tet4(cell_nodes.shape[0], _p(coords), _p(cell_nodes), _p(fv), _p(rhs))
    return rhs


def rhs_constant_source_q1(dim, coords, cell_nodes, nc_ptr, nc_cell, qdot, nb_dof=1):
    coords = _c(coords, np.float64)
    cell_nodes = _c(cell_nodes, np.int32)
    rhs = np.zeros(coords.shape[0] * nb_dof)
    lib().afo_rhs_constant_source_q1(dim, coords.shape[0], _p(coords), _p(cell_nodes), _p(_c(nc_ptr, np.int32)),
                                     _p(_c(nc_cell, np.int32)), float(qdot), nb_dof, _p(rhs))
    return rhs


FACE_SCALAR, FACE_NORMAL, FACE_VECTOR = 0, 1, 2


def rhs_boundary_faces(dim, coords, face_nodes, outward, mode, g, nb_dof, rhs):
    """Neumann (scalar / normal flux) or traction terms of boundary faces, += into rhs."""
    coords = _c(coords, np.float64)
    face_nodes = _c(face_nodes, np.int32)
    out = None if outward is None else _c(outward, np.uint8)
    gv = _c(np.resize(np.asarray(g, np.float64), 3), np.float64)
    lib().afo_rhs_boundary_faces(dim, face_nodes.shape[0], _p(coords), _p(face_nodes), _p(out), mode, _p(gv),
                                 nb_dof, _p(rhs))
    return rhs


def dirichlet_penalty(nodes, nb_dof, dof_index, value, penalty, forced_info, forced_value, rhs):
    nodes = _c(nodes, np.int32)
    lib().afo_dirichlet_penalty(nodes.size, _p(nodes), nb_dof, dof_index, value, penalty, _p(forced_info),
                                _p(forced_value), _p(rhs))


def dirichlet_elimination(nodes, nb_dof, dof_index, value, elim_type, elim_info, elim_value):
    nodes = _c(nodes, np.int32)
    lib().afo_dirichlet_elimination(nodes.size, _p(nodes), nb_dof, dof_index, value, elim_type, _p(elim_info),
                                    _p(elim_value))


def apply_transformations(row_ptr, cols, values, rhs, forced_info, forced_value, elim_info, elim_value):
    """applyMatrixTransformation then applyRHSTransformation, in place on values and rhs."""
    n = row_ptr.size - 1
    nnz = int(row_ptr[-1])
    rc_saved = np.zeros(nnz)
    rc_mask = np.zeros(nnz, np.uint8)
    rp, cl = _c(row_ptr, np.int32), _c(cols, np.int32)
    L = lib()
    L.afo_apply_matrix_transformation(n, _p(rp), _p(cl), _p(values), _p(forced_info), _p(forced_value),
                                      _p(elim_info), _p(elim_value), _p(rc_saved), _p(rc_mask))
    L.afo_apply_rhs_transformation(n, _p(rp), _p(cl), _p(elim_info), _p(elim_value), _p(rc_saved), _p(rc_mask),
                                   _p(rhs))


def spmv(row_ptr, cols, values, x):
    y = np.zeros(row_ptr.size - 1)
    lib().afo_spmv(row_ptr.size - 1, _p(_c(row_ptr, np.int32)), _p(_c(cols, np.int32)), _p(_c(values, np.float64)),
                   _p(_c(x, np.float64)), _p(y))
    return y


def pcg_jacobi(row_ptr, cols, values, b, rtol=1e-12, max_iter=100000, x0=None, norm_skip=None, nb_threads=1):
    n = row_ptr.size - 1
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    relres = C.c_double(0.0)
    skip = None if norm_skip is None else _c(norm_skip, np.uint8)
    it = lib().afo_pcg_jacobi(n, _p(_c(row_ptr, np.int32)), _p(_c(cols, np.int32)), _p(_c(values, np.float64)),
                              _p(_c(b, np.float64)), _p(x), rtol, max_iter, _p(skip), C.byref(relres),
                              int(nb_threads))
    return x, int(it), float(relres.value)


def assemble_dok(kind, nb_node, coords, cell_nodes, nb_cell=None):
    """The reference's DOK assembly (ordered (row, col) map, zeros skipped) of
    the first nb_cell cells, as CSR (row_ptr, cols, values).  Poisson P1."""
    cn = _c(cell_nodes, np.int32)
    nc = cn.shape[0] if nb_cell is None else int(nb_cell)
    cap = nc * cn.shape[1] ** 2
    rp = np.zeros(nb_node + 1, np.int32)
    cols = np.zeros(max(cap, 1), np.int32)
    vals = np.zeros(max(cap, 1))
    nnz = lib().afo_assemble_dok(kind, nb_node, nc, _p(_c(coords, np.float64)), _p(cn), _p(rp), _p(cols), _p(vals),
                                 cap)
    assert nnz >= 0
    return rp, cols[:nnz].copy(), vals[:nnz].copy()


def sparsity_nodewise(nb_node, cell_nodes, nc_ptr, nc_cell, nb_threads=1):
    """Node-wise sparsity (ascending columns) on nb_threads threads."""
    cn = _c(cell_nodes, np.int32)
    rp = np.zeros(nb_node + 1, np.int32)
    cap = int(np.diff(nc_ptr).sum()) * cn.shape[1] + nb_node
    cols = np.zeros(cap, np.int32)
    nnz = lib().afo_sparsity_nodewise(nb_node, cn.shape[1], _p(cn), _p(_c(nc_ptr, np.int32)),
                                      _p(_c(nc_cell, np.int32)), _p(rp), _p(cols), cap, int(nb_threads))
    assert nnz >= 0
    return rp, cols[:nnz].copy()


def wtime() -> float:
    return float(lib().afo_wtime())
