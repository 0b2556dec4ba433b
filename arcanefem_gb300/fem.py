"""Host-side mirror of ArcaneFEM's assembly and linear-system interfaces.

Names and argument meanings follow the reference so that code written
against it reads the same:

* :class:`BSRFormat` mirrors ``femutils/BSRFormat.h:157-249``
  (``initialize``, ``computeSparsity``, ``assembleBilinear*``,
  ``toLinearSystem``, ``matrix``, ``resetMatrixValues``), node-wise
  (atomic-free) only.
* :class:`DoFLinearSystem` mirrors the facade of
  ``femutils/DoFLinearSystem.h:154-409`` over the CSR implementation
  (``internal/CsrDoFLinearSystemImpl.h``): ``setCSRValues``,
  ``applyMatrixTransformation``, ``applyRHSTransformation``, ``solve``,
  ``rhsVariable``, ``solutionVariable``, forced / elimination variables.
* Dirichlet helpers mirror ``Gpu::BoundaryConditions``
  (``femutils/ArcaneFemFunctionsGpu.cc:54-147``).

Every operation runs in libafem_gb300.so on the GPU (PyTorch only supplies
device memory and the stream).  Errors surface as :class:`AfemError`, the
counterpart of the reference's ARCANE_FATAL / ARCANE_THROW.
"""
from __future__ import annotations

import ctypes as C
import sys
import weakref
from dataclasses import dataclass

import torch

from . import _capi
from ._capi import (AfemError, COLS_ASCENDING, COLS_SELF_LAST, ELIMINATE_ROW, ELIMINATE_ROW_COLUMN,  # noqa: F401
                    FORMULATION_MINIMAL, FORMULATION_REFERENCE, FORMULATION_TESTLAB, LAYOUT_PER_BLOCK,
                    LAYOUT_PER_ROW, PRECISION_FP64, PRECISION_MIXED, PRECOND_JACOBI, PRECOND_LEARNED, PRECOND_NONE,
                    MeshView, SolveInfo, SolverOptions, call)


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(0 if t is None else t.data_ptr())


def solve_call(name: str, info: SolveInfo, *args) -> SolveInfo:
    """Call a solver entry point; on a failure status (not converged, breakdown)
    the raised AfemError carries the filled SolveInfo as ``.info`` (the
    solution argument then holds the last iterate)."""
    try:
        call(name, *args)
    except AfemError as e:
        e.info = info
        raise
    return info


class _DeviceArray:
    """Zero-copy view of library-owned device memory (__cuda_array_interface__)."""

    def __init__(self, ptr: int, shape, typestr: str):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def device_view(ptr: int, n: int, dtype) -> torch.Tensor:
    typestr = {torch.float64: "<f8", torch.uint8: "|u1", torch.int32: "<i4"}[dtype]
    return torch.as_tensor(_DeviceArray(ptr, (n,), typestr), device="cuda")


class Context:
    """A stream plus the library's scratch arena (the reference's RunQueue)."""

    def __init__(self, stream: torch.cuda.Stream | None = None):
        self.stream = stream or torch.cuda.current_stream()
        h = C.c_void_p()
        call("afem_context_create", C.byref(h), C.c_void_p(self.stream.cuda_stream))
        self.handle = h
        # handles created on this context (linear systems, networks, batches):
        # closed before it, since the library's objects use their context's stream
        self._children = weakref.WeakSet()

    def adopt(self, child) -> None:
        """Register an object with a close() that must run before the context's."""
        self._children.add(child)

    def synchronize(self) -> None:
        """Wait for the stream; raises AFEM_ERR_MESH if an element kernel met a degenerate cell."""
        call("afem_context_synchronize", self.handle)

    @property
    def formulation(self) -> int:
        """Element arithmetic of the assembly kernels: FORMULATION_REFERENCE (default, bit-identical
        to the reference), FORMULATION_TESTLAB or FORMULATION_MINIMAL (fewest FP64 instructions)."""
        v = C.c_int()
        call("afem_context_get_element_formulation", self.handle, C.byref(v))
        return int(v.value)

    @formulation.setter
    def formulation(self, f: int) -> None:
        call("afem_context_set_element_formulation", self.handle, int(f))

    @property
    def launches(self) -> int:
        v = C.c_int64()
        call("afem_context_launch_count", self.handle, C.byref(v))
        return int(v.value)

    def fp64_fma_rate(self) -> float:
        """Measured FP64 FMA issue rate of the device, in G FMA/s."""
        v = C.c_double()
        call("afem_device_fp64_fma_rate", self.handle, C.byref(v))
        return float(v.value)

    def close(self) -> None:
        if self.handle:
            for child in list(self._children):
                child.close()
            call("afem_context_destroy", self.handle)
            self.handle = None

    def __del__(self):
        # at interpreter shutdown the CUDA runtime may already be torn down: leak instead
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Mesh:
    """Device-resident P1 mesh: coords float64 [N, 3], cells int32 [C, dim+1]."""
    dim: int
    coords: torch.Tensor
    cells: torch.Tensor

    @staticmethod
    def from_host(dim, coords, cells, device="cuda") -> "Mesh":
        co = torch.as_tensor(coords, dtype=torch.float64).contiguous().to(device)
        ce = torch.as_tensor(cells, dtype=torch.int32).contiguous().to(device)
        return Mesh(dim, co, ce)

    @property
    def nb_node(self) -> int:
        return int(self.coords.shape[0])

    @property
    def nb_cell(self) -> int:
        return int(self.cells.shape[0])

    @property
    def npc(self) -> int:
        return int(self.cells.shape[1])


class BSRFormat:
    """Node-wise (atomic-free) block sparse row assembly: BSRFormat with
    ``use_atomic_free = true`` (femutils/BSRFormat.cc:350-372)."""

    def __init__(self, ctx: Context, mesh: Mesh):
        self.ctx = ctx
        self.mesh = mesh
        self.nb_dof = 1
        self.order_values_per_block = False
        self.col_order = COLS_ASCENDING
        self.nc_ptr = self.nc_cell = self.nc_local = self.nc_slot = None
        self.row_ptr = self.cols = self.values = None
        self.nnzb = 0

    # BSRFormat::initialize(mesh, nb_dof, does_linear_system_use_csr, use_atomic_free)
    def initialize(self, nb_dof: int, does_linear_system_use_csr: bool = True, col_order: int = COLS_ASCENDING):
        if nb_dof not in (1, 3) or (nb_dof == 3 and self.mesh.dim != 3):
            raise AfemError(1, "BSRFormat.initialize: nb_dof must be 1, or 3 on tetrahedra")
        self.nb_dof = nb_dof
        self.order_values_per_block = not does_linear_system_use_csr
        self.col_order = col_order
        m = self.mesh
        dev = m.coords.device
        total = m.nb_cell * m.npc
        self.nc_ptr = torch.empty(m.nb_node + 1, dtype=torch.int32, device=dev)
        self.nc_cell = torch.empty(total, dtype=torch.int32, device=dev)
        self.nc_local = torch.empty(total, dtype=torch.uint8, device=dev)
        self.nc_inverse = torch.empty(total, dtype=torch.int32, device=dev)
        call("afem_node_cell_build", self.ctx.handle, m.nb_node, m.nb_cell, m.npc, _ptr(m.cells), _ptr(self.nc_ptr),
             _ptr(self.nc_cell), _ptr(self.nc_local), _ptr(self.nc_inverse))

    # BSRFormat::computeSparsity (femutils/BSRFormat.cc:1011-1018)
    def compute_sparsity(self):
        m = self.mesh
        dev = m.coords.device
        self.row_ptr = torch.empty(m.nb_node + 1, dtype=torch.int32, device=dev)
        nnz = C.c_int64()
        call("afem_sparsity_rows", self.ctx.handle, m.nb_node, m.npc, _ptr(m.cells), _ptr(self.nc_ptr),
             _ptr(self.nc_cell), _ptr(self.row_ptr), C.byref(nnz))
        self.nnzb = int(nnz.value)
        self.cols = torch.empty(self.nnzb, dtype=torch.int32, device=dev)
        self.nc_slot = torch.empty(m.nb_cell * m.npc * m.npc, dtype=torch.uint8, device=dev)
        call("afem_sparsity_cols", self.ctx.handle, m.nb_node, m.npc, _ptr(m.cells), _ptr(self.nc_ptr),
             _ptr(self.nc_cell), _ptr(self.nc_local), _ptr(self.row_ptr), self.col_order, _ptr(self.cols),
             _ptr(self.nc_slot))
        self.values = torch.zeros(self.nnzb * self.nb_dof ** 2, dtype=torch.float64, device=dev)

    def mesh_view(self) -> MeshView:
        m = self.mesh
        return MeshView(m.dim, m.nb_node, m.nb_cell, m.coords.data_ptr(), m.cells.data_ptr(), self.nc_ptr.data_ptr(),
                        self.nc_cell.data_ptr(), self.nc_local.data_ptr(),
                        0 if self.nc_slot is None else self.nc_slot.data_ptr(), self.nc_inverse.data_ptr())

    # assembleBilinearAtomicFree with the Poisson element vectors
    def is_q1(self) -> bool:
        """Quad4 / Hexa8 cells (2^dim nodes) rather than P1 simplices."""
        return self.mesh.npc == 1 << self.mesh.dim

    def assemble_poisson(self, cell_coeff: torch.Tensor | None = None):
        mv = self.mesh_view()
        fn = "afem_assemble_poisson_q1" if self.is_q1() else "afem_assemble_poisson_p1"
        call(fn, self.ctx.handle, C.byref(mv), _ptr(self.row_ptr), _ptr(cell_coeff), _ptr(self.values))

    # assembleBilinearAtomicFree with the elasticity element vectors (Lame lambda, mu)
    def assemble_elasticity(self, lam: float, mu: float):
        mv = self.mesh_view()
        layout = LAYOUT_PER_BLOCK if self.order_values_per_block else LAYOUT_PER_ROW
        call("afem_assemble_elasticity_tet4", self.ctx.handle, C.byref(mv), _ptr(self.row_ptr), float(lam), float(mu),
             layout, _ptr(self.values))

    def element_buffer_size(self) -> int:
        """Doubles of the stage-1 element rows (incidence order): npc^2 per cell, 144 for elasticity."""
        per_cell = 144 if self.nb_dof == 3 else self.mesh.npc ** 2
        return per_cell * self.mesh.nb_cell

    # the two stages of assemble_poisson / assemble_elasticity, caller-owned element matrices
    def element_matrices(self, ke: torch.Tensor, cell_coeff: torch.Tensor | None = None, lam=0.0, mu=0.0):
        mv = self.mesh_view()
        if self.nb_dof == 3:
            call("afem_element_matrices_elasticity_tet4", self.ctx.handle, C.byref(mv), float(lam), float(mu), _ptr(ke))
        else:
            fn = "afem_element_matrices_poisson_q1" if self.is_q1() else "afem_element_matrices_poisson_p1"
            call(fn, self.ctx.handle, C.byref(mv), _ptr(cell_coeff), _ptr(ke))

    def gather(self, ke: torch.Tensor):
        mv = self.mesh_view()
        if self.nb_dof == 3:
            layout = LAYOUT_PER_BLOCK if self.order_values_per_block else LAYOUT_PER_ROW
            call("afem_gather_elasticity_tet4", self.ctx.handle, C.byref(mv), _ptr(self.row_ptr), _ptr(ke), layout,
                 _ptr(self.values))
        else:
            fn = "afem_gather_poisson_q1" if self.is_q1() else "afem_gather_poisson_p1"
            call(fn, self.ctx.handle, C.byref(mv), _ptr(self.row_ptr), _ptr(ke), _ptr(self.values))

    def gather_to_host(self, ke: torch.Tensor, values_h: torch.Tensor, chunks: int = 0):
        """gather() with the values copied into the host tensor values_h
        (pinned for overlap) range by range while the next range is gathered;
        returns when values_h is complete.  chunks = 0: one range per ~80 MB
        of values (at most 12)."""
        assert values_h.device.type == "cpu" and values_h.dtype == torch.float64
        assert values_h.numel() == self.values.numel() and values_h.is_contiguous()
        mv = self.mesh_view()
        layout = 0
        if self.nb_dof == 3:
            kind = GATHER_ELASTICITY_TET4
            layout = LAYOUT_PER_BLOCK if self.order_values_per_block else LAYOUT_PER_ROW
        else:
            kind = GATHER_POISSON_Q1 if self.is_q1() else GATHER_POISSON_P1
        call("afem_gather_to_host", self.ctx.handle, C.byref(mv), kind, _ptr(self.row_ptr), _ptr(ke), layout,
             _ptr(self.values), C.c_void_p(values_h.data_ptr()), int(chunks))

    def assemble_to_host(self, ke: torch.Tensor, values_h: torch.Tensor, chunks: int = 0,
                         cell_coeff: torch.Tensor | None = None, lam=0.0, mu=0.0, coords_h: torch.Tensor | None = None):
        """element_matrices + gather with the values copied into the host
        tensor values_h (pinned for overlap), the copies overlapping the
        element computation of later cell ranges (P1 and Q1 Poisson, P1
        elasticity).  chunks = 0: one range per ~80 MB of values (at most 12).
        With coords_h (host [nb_node, 3] float64, pinned for overlap) the node
        coordinates are uploaded into the mesh's device coordinates in node
        prefixes, each ahead of the first cell range that uses it."""
        assert values_h.device.type == "cpu" and values_h.dtype == torch.float64
        assert values_h.numel() == self.values.numel() and values_h.is_contiguous()
        mv = self.mesh_view()
        if self.nb_dof == 3:
            kind = GATHER_ELASTICITY_TET4
            layout = LAYOUT_PER_BLOCK if self.order_values_per_block else LAYOUT_PER_ROW
        else:
            kind, layout = (GATHER_POISSON_Q1 if self.is_q1() else GATHER_POISSON_P1), 0
        if coords_h is not None:
            assert coords_h.device.type == "cpu" and coords_h.dtype == torch.float64 and coords_h.is_contiguous()
            assert coords_h.numel() == 3 * self.mesh.nb_node
            call("afem_assemble_host_io", self.ctx.handle, C.byref(mv), C.c_void_p(coords_h.data_ptr()), kind,
                 _ptr(self.row_ptr), _ptr(cell_coeff), float(lam), float(mu), layout, _ptr(ke), _ptr(self.values),
                 C.c_void_p(values_h.data_ptr()), int(chunks))
            return
        call("afem_assemble_to_host", self.ctx.handle, C.byref(mv), kind, _ptr(self.row_ptr), _ptr(cell_coeff),
             float(lam), float(mu), layout, _ptr(ke), _ptr(self.values), C.c_void_p(values_h.data_ptr()), int(chunks))

    def reset_matrix_values(self):
        self.values.zero_()

    # BSRMatrix::toCsr on the device (femutils/BSRFormat.cc:110-172)
    def to_csr(self):
        if self.nb_dof == 1:
            return self.row_ptr, self.cols, self.values
        if self.order_values_per_block:
            raise AfemError(1, "to_csr needs the per-row (CSR-compatible) value layout")
        b = self.nb_dof
        m = self.mesh
        rp = torch.empty(m.nb_node * b + 1, dtype=torch.int32, device=self.row_ptr.device)
        cl = torch.empty(self.nnzb * b * b, dtype=torch.int32, device=self.row_ptr.device)
        call("afem_bsr_to_csr_structure", self.ctx.handle, m.nb_node, b, _ptr(self.row_ptr), _ptr(self.cols), _ptr(rp),
             _ptr(cl))
        return rp, cl, self.values

    # BSRFormat::toLinearSystem (CSR path)
    def to_linear_system(self, ls: "DoFLinearSystem"):
        rp, cl, v = self.to_csr()
        ls.set_csr_values(rp, cl, v)
        ls.block_size = self.nb_dof   # the scalar rows come in nb_dof x nb_dof blocks
        return rp, cl, v

    def rhs_constant_source(self, qdot: float, rhs: torch.Tensor):
        mv = self.mesh_view()
        fn = "afem_rhs_constant_source_q1" if self.is_q1() else "afem_rhs_constant_source"
        call(fn, self.ctx.handle, C.byref(mv), float(qdot), self.nb_dof, _ptr(rhs))

    def rhs_body_force(self, f, rhs: torch.Tensor):
        mv = self.mesh_view()
        call("afem_rhs_body_force_tet4", self.ctx.handle, C.byref(mv), float(f[0]), float(f[1]), float(f[2]),
             _ptr(rhs))


GATHER_POISSON_P1, GATHER_POISSON_Q1, GATHER_ELASTICITY_TET4 = 0, 1, 2


def solver_options(rtol=1e-7, atol=0.0, max_iter=1000, precond=PRECOND_JACOBI, precision=PRECISION_FP64,
                   skip_forced_rows=False, inner_rtol=0.0, check_every=16, block_size=0) -> SolverOptions:
    return SolverOptions(rtol, atol, max_iter, precond, precision, int(skip_forced_rows), inner_rtol, check_every,
                         block_size)


class DoFLinearSystem:
    """CSR linear system on the device (CsrDoFLinearSystemImpl semantics)."""

    def __init__(self, ctx: Context, nb_dof: int):
        self.ctx = ctx
        self.n = nb_dof
        h = C.c_void_p()
        call("afem_ls_create", ctx.handle, nb_dof, C.byref(h))
        self.handle = h
        ctx.adopt(self)
        ptrs = [C.c_void_p() for _ in range(6)]
        call("afem_ls_dof_variables", h, *[C.byref(p) for p in ptrs])
        self._rhs = device_view(ptrs[0].value, nb_dof, torch.float64)
        self._sol = device_view(ptrs[1].value, nb_dof, torch.float64)
        self._fi = device_view(ptrs[2].value, nb_dof, torch.uint8)
        self._fv = device_view(ptrs[3].value, nb_dof, torch.float64)
        self._ei = device_view(ptrs[4].value, nb_dof, torch.uint8)
        self._ev = device_view(ptrs[5].value, nb_dof, torch.float64)
        self._keep = None

    def rhs_variable(self) -> torch.Tensor:
        return self._rhs

    def solution_variable(self) -> torch.Tensor:
        return self._sol

    def get_forced_info(self) -> torch.Tensor:
        return self._fi

    def get_forced_value(self) -> torch.Tensor:
        return self._fv

    def get_elimination_info(self) -> torch.Tensor:
        return self._ei

    def get_elimination_value(self) -> torch.Tensor:
        return self._ev

    def has_set_csr_values(self) -> bool:
        return True

    def set_csr_values(self, row_ptr: torch.Tensor, cols: torch.Tensor, values: torch.Tensor):
        self._keep = (row_ptr, cols, values)   # the view is non-owning: keep the tensors alive
        call("afem_ls_set_csr_values", self.handle, _ptr(row_ptr), _ptr(cols), _ptr(values), int(cols.numel()))

    def set_csr_view(self, rows: torch.Tensor, columns: torch.Tensor, values: torch.Tensor,
                     rows_nb_column: torch.Tensor | None = None):
        """setCSRValues with the reference's CsrFormatMatrixView layout: `rows` holds
        one start per row (no trailing entry, the last row ends at columns.numel()),
        `columns` may hold -1 in unused slots; `rows_nb_column` (optional) the slot
        count of each row.  Non-owning, like set_csr_values."""
        self._keep = (rows, columns, values, rows_nb_column)   # non-owning view: keep the tensors alive
        call("afem_ls_set_csr_view", self.handle, int(rows.numel()), _ptr(rows), _ptr(rows_nb_column),
             int(columns.numel()), _ptr(columns), _ptr(values))

    def set_learned_preconditioner(self, net):
        """Attach the learned preconditioner (a learned.MPNN built on this system's
        matrix graph) for solves with precond = PRECOND_LEARNED; None detaches it."""
        self._learned = net
        call("afem_ls_set_learned_preconditioner", self.handle, None if net is None else net.handle)

    def clear_values(self):
        call("afem_ls_clear_values", self.handle)
        self._keep = None

    def matrix_add_value(self, row: int, col: int, value: float):
        call("afem_ls_matrix_add_value", self.handle, int(row), int(col), float(value))

    def matrix_set_value(self, row: int, col: int, value: float):
        call("afem_ls_matrix_set_value", self.handle, int(row), int(col), float(value))

    def eliminate_row(self, row: int, value: float):
        call("afem_ls_eliminate_row", self.handle, int(row), float(value))

    def eliminate_row_column(self, row: int, value: float):
        call("afem_ls_eliminate_row_column", self.handle, int(row), float(value))

    def apply_matrix_transformation(self):
        call("afem_ls_apply_matrix_transformation", self.handle)

    def apply_rhs_transformation(self):
        call("afem_ls_apply_rhs_transformation", self.handle)

    def solve(self, options: SolverOptions | None = None) -> SolveInfo:
        """Solve; a system filled from a 3-DoF BSRFormat passes its block size
        to the mixed-precision solver (FP32 BSR SpMV) unless the options set one."""
        info = SolveInfo()
        opt = options or solver_options()
        if opt.block_size == 0 and getattr(self, "block_size", 1) == 3:
            opt = SolverOptions.from_buffer_copy(opt)
            opt.block_size = 3
        return solve_call("afem_ls_solve", info, self.handle, C.byref(opt), C.byref(info))

    # DoFLinearSystem::applyLinearSystemTransformationAndSolve (DoFLinearSystem.cc:487-493)
    def apply_linear_system_transformation_and_solve(self, options: SolverOptions | None = None) -> SolveInfo:
        self.apply_matrix_transformation()
        self.apply_rhs_transformation()
        return self.solve(options)

    # Gpu::BoundaryConditions helpers (ArcaneFemFunctionsGpu.cc:54-105)
    def apply_dirichlet_penalty(self, nodes: torch.Tensor, nb_dof_per_node: int, dof_index: int, value: float,
                                penalty: float = 1e30):
        call("afem_dirichlet_penalty", self.handle, int(nodes.numel()), _ptr(nodes), nb_dof_per_node, dof_index,
             float(value), float(penalty))

    def apply_dirichlet_elimination(self, elimination_type: int, nodes: torch.Tensor, nb_dof_per_node: int,
                                    dof_index: int, value: float):
        call("afem_dirichlet_elimination", self.handle, int(elimination_type), int(nodes.numel()), _ptr(nodes),
             nb_dof_per_node, dof_index, float(value))

    def close(self):
        if self.handle:
            call("afem_ls_destroy", self.handle)
            self.handle = None

    def __del__(self):
        if sys.is_finalizing():
            return
        try:
            self.close()
        except Exception:
            pass


def cg_solve_csr(ctx: Context, row_ptr, cols, values, b, x, forced_info=None, options: SolverOptions | None = None):
    info = SolveInfo()
    opt = options or solver_options()
    n = int(row_ptr.numel()) - 1
    return solve_call("afem_cg_solve_csr", info, ctx.handle, n, _ptr(row_ptr), _ptr(cols), _ptr(values), _ptr(b),
                      _ptr(x), _ptr(forced_info), C.byref(opt), C.byref(info))


FACE_SCALAR, FACE_NORMAL, FACE_VECTOR = 0, 1, 2


def rhs_boundary_faces(ctx: Context, dim: int, coords, face_nodes, outward, mode: int, g, nb_dof: int, rhs):
    """Neumann flux (scalar or normal) or traction of boundary faces added into
    rhs: applyNeumannToRhsTria3/Tetra4 and applyTractionToRhsTria3/Tetra4 with
    a deterministic node-wise gather (see afem_rhs_boundary_faces)."""
    gv = (C.c_double * 3)(*([float(v) for v in g] + [0.0] * (3 - len(g))))
    call("afem_rhs_boundary_faces", ctx.handle, dim, int(coords.shape[0]), int(face_nodes.shape[0]), _ptr(coords),
         _ptr(face_nodes), _ptr(outward), mode, gv, nb_dof, _ptr(rhs))


def spmv_csr(ctx: Context, row_ptr, cols, values, x, y):
    call("afem_spmv_csr", ctx.handle, int(row_ptr.numel()) - 1, _ptr(row_ptr), _ptr(cols), _ptr(values), _ptr(x),
         _ptr(y))


def lame(E: float, nu: float):
    """Lame parameters as modules/elasticity/FemModule.cc:171-172."""
    mu = E / (2 * (1 + nu))
    lam = E * nu / ((1 + nu) * (1 - 2 * nu))
    return lam, mu
