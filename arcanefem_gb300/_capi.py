"""ctypes binding of libafem_gb300.so (the C ABI declared in include/afem_gb300.h).

The library is the product: there is no Python or CPU fallback.  Loading
fails loudly when the shared object is missing (build it with
``python -c "import __graft_entry__ as g; g.build()"``).
"""
from __future__ import annotations

import ctypes as C
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib", "libafem_gb300.so")

AFEM_OK = 0
NOT_CONVERGED = 3
STATUS_NAMES = {0: "AFEM_OK", 1: "AFEM_ERR_BAD_ARG", 2: "AFEM_ERR_OOM", 3: "AFEM_ERR_NOT_CONVERGED",
                4: "AFEM_ERR_BREAKDOWN", 5: "AFEM_ERR_TIMEOUT", 6: "AFEM_ERR_CUDA", 7: "AFEM_ERR_MESH",
                8: "AFEM_ERR_NOT_IMPLEMENTED", 9: "AFEM_ERR_NOT_FOUND"}
COLS_ASCENDING, COLS_SELF_LAST = 0, 1
LAYOUT_PER_BLOCK, LAYOUT_PER_ROW = 0, 1
ELIMINATE_NONE, ELIMINATE_ROW, ELIMINATE_ROW_COLUMN = 0, 1, 2
PRECOND_NONE, PRECOND_JACOBI, PRECOND_LEARNED = 0, 1, 2
PRECISION_FP64, PRECISION_MIXED = 0, 1
FORMULATION_REFERENCE, FORMULATION_TESTLAB, FORMULATION_MINIMAL = 0, 1, 2


class AfemError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class MeshView(C.Structure):
    _fields_ = [("dim", C.c_int), ("nb_node", C.c_int), ("nb_cell", C.c_int), ("coords_d", C.c_void_p),
                ("cell_nodes_d", C.c_void_p), ("nc_ptr_d", C.c_void_p), ("nc_cell_d", C.c_void_p),
                ("nc_local_d", C.c_void_p), ("nc_slot_d", C.c_void_p), ("nc_inverse_d", C.c_void_p)]


class SolverOptions(C.Structure):
    _fields_ = [("rtol", C.c_double), ("atol", C.c_double), ("max_iter", C.c_int), ("precond", C.c_int),
                ("precision", C.c_int), ("skip_forced_rows", C.c_int), ("inner_rtol", C.c_double),
                ("check_every", C.c_int), ("block_size", C.c_int)]


class SolveInfo(C.Structure):
    _fields_ = [("iterations", C.c_int), ("refinements", C.c_int), ("status", C.c_int), ("relres", C.c_double),
                ("solve_ms", C.c_double)]


_P = C.c_void_p
_PP = C.POINTER(C.c_void_p)
_I64P = C.POINTER(C.c_int64)

# name -> (restype, argtypes)
SIGNATURES = {
    "afem_last_error": (C.c_char_p, []),
    "afem_version": (C.c_int, []),
    "afem_context_create": (C.c_int, [_PP, _P]),
    "afem_context_destroy": (C.c_int, [_P]),
    "afem_context_set_stream": (C.c_int, [_P, _P]),
    "afem_context_synchronize": (C.c_int, [_P]),
    "afem_context_launch_count": (C.c_int, [_P, _I64P]),
    "afem_context_set_element_formulation": (C.c_int, [_P, C.c_int]),
    "afem_context_get_element_formulation": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "afem_device_fp64_fma_rate": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "afem_node_cell_build": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P, _P, _P, _P]),
    "afem_sparsity_rows": (C.c_int, [_P, C.c_int, C.c_int, _P, _P, _P, _P, _I64P]),
    "afem_sparsity_cols": (C.c_int, [_P, C.c_int, C.c_int, _P, _P, _P, _P, _P, C.c_int, _P, _P]),
    "afem_assemble_poisson_p1": (C.c_int, [_P, C.POINTER(MeshView), _P, _P, _P]),
    "afem_assemble_elasticity_tet4": (C.c_int, [_P, C.POINTER(MeshView), _P, C.c_double, C.c_double, C.c_int,
                                                _P]),
    "afem_element_matrices_poisson_p1": (C.c_int, [_P, C.POINTER(MeshView), _P, _P]),
    "afem_gather_poisson_p1": (C.c_int, [_P, C.POINTER(MeshView), _P, _P, _P]),
    "afem_assemble_poisson_q1": (C.c_int, [_P, C.POINTER(MeshView), _P, _P, _P]),
    "afem_element_matrices_poisson_q1": (C.c_int, [_P, C.POINTER(MeshView), _P, _P]),
    "afem_gather_poisson_q1": (C.c_int, [_P, C.POINTER(MeshView), _P, _P, _P]),
    "afem_rhs_constant_source_q1": (C.c_int, [_P, C.POINTER(MeshView), C.c_double, C.c_int, _P]),
    "afem_assemble_poisson_p1_noalloc": (C.c_int, [_P, C.POINTER(MeshView), _P, _P, _P]),
    "afem_element_matrices_elasticity_tet4": (C.c_int, [_P, C.POINTER(MeshView), C.c_double, C.c_double, _P]),
    "afem_gather_elasticity_tet4": (C.c_int, [_P, C.POINTER(MeshView), _P, _P, C.c_int, _P]),
    "afem_gather_to_host": (C.c_int, [_P, C.POINTER(MeshView), C.c_int, _P, _P, C.c_int, _P, _P, C.c_int]),
    "afem_assemble_to_host": (C.c_int, [_P, C.POINTER(MeshView), C.c_int, _P, _P, C.c_double, C.c_double, C.c_int,
                                        _P, _P, _P, C.c_int]),
    "afem_assemble_host_io": (C.c_int, [_P, C.POINTER(MeshView), _P, C.c_int, _P, _P, C.c_double, C.c_double,
                                        C.c_int, _P, _P, _P, C.c_int]),
    "afem_bsr_to_csr_structure": (C.c_int, [_P, C.c_int, C.c_int, _P, _P, _P, _P]),
    "afem_rhs_constant_source": (C.c_int, [_P, C.POINTER(MeshView), C.c_double, C.c_int, _P]),
    "afem_rhs_body_force_tet4": (C.c_int, [_P, C.POINTER(MeshView), C.c_double, C.c_double, C.c_double, _P]),
    "afem_ls_create": (C.c_int, [_P, C.c_int, _PP]),
    "afem_ls_destroy": (C.c_int, [_P]),
    "afem_ls_set_csr_values": (C.c_int, [_P, _P, _P, _P, C.c_int64]),
    "afem_ls_get_csr_values": (C.c_int, [_P, _PP, _PP, _PP, _I64P]),
    "afem_ls_set_csr_view": (C.c_int, [_P, C.c_int32, _P, _P, C.c_int64, _P, _P]),
    "afem_ls_dof_variables": (C.c_int, [_P, _PP, _PP, _PP, _PP, _PP, _PP]),
    "afem_ls_clear_values": (C.c_int, [_P]),
    "afem_ls_matrix_add_value": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_double]),
    "afem_ls_matrix_set_value": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_double]),
    "afem_ls_eliminate_row": (C.c_int, [_P, C.c_int32, C.c_double]),
    "afem_ls_eliminate_row_column": (C.c_int, [_P, C.c_int32, C.c_double]),
    "afem_dirichlet_penalty": (C.c_int, [_P, C.c_int, _P, C.c_int, C.c_int, C.c_double, C.c_double]),
    "afem_dirichlet_elimination": (C.c_int, [_P, C.c_int, C.c_int, _P, C.c_int, C.c_int, C.c_double]),
    "afem_ls_apply_matrix_transformation": (C.c_int, [_P]),
    "afem_ls_apply_rhs_transformation": (C.c_int, [_P]),
    "afem_solver_options_default": (None, [C.POINTER(SolverOptions)]),
    "afem_cg_solve_csr": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _P, _P, C.POINTER(SolverOptions),
                                    C.POINTER(SolveInfo)]),
    "afem_ls_solve": (C.c_int, [_P, C.POINTER(SolverOptions), C.POINTER(SolveInfo)]),
    "afem_ls_set_learned_preconditioner": (C.c_int, [_P, _P]),
    "afem_spmv_csr": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _P]),
    "afem_mpnn_create": (C.c_int, None),
    "afem_mpnn_destroy": (C.c_int, [_P]),
    "afem_mpnn_param_count": (C.c_int, [_P]),
    "afem_mpnn_set_params": (C.c_int, [_P, _P]),
    "afem_mpnn_get_params": (C.c_int, [_P, _P]),
    "afem_mpnn_set_operator": (C.c_int, [_P, C.c_int, _P, _P, _P]),
    "afem_mpnn_forward": (C.c_int, [_P, C.c_int, _P, _P]),
    "afem_mpnn_scalings": (C.c_int, [_P, C.c_int, _P]),
    "afem_mpnn_set_coarse_rows": (C.c_int, [_P, C.c_int]),
    "afem_mpnn_gradients": (C.c_int, [_P, C.c_int, _P, _P, _P, C.POINTER(C.c_double)]),
    "afem_mpnn_train_step": (C.c_int, [_P, C.c_int, _P, _P, C.c_float, C.POINTER(C.c_double)]),
    "afem_tc_row_gemm": (C.c_int, [_P, C.c_int64, _P, _P, _P, _P, _P, C.c_int, _P, _P, C.c_int]),
    "afem_tc_weight_grad": (C.c_int, [_P, C.c_int64, _P, _P, _P, _P]),
    "afem_fcg_solve": (C.c_int, [_P, C.c_int, _P, _P, _P, _P, _P, _P, C.POINTER(SolverOptions),
                                 C.POINTER(SolveInfo)]),
    "afem_rhs_boundary_faces": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, _P, _P, C.c_int,
                                          C.POINTER(C.c_double), C.c_int, _P]),
    "afem_batch_create": (C.c_int, None),
    "afem_batch_destroy": (C.c_int, [_P]),
    "afem_batch_set_config": (C.c_int, None),
    "afem_batch_get_config": (C.c_int, None),
    "afem_batch_team": (C.c_int, None),
    "afem_batch_set_weights": (C.c_int, None),
    "afem_batch_solve": (C.c_int, None),
    "afem_batch_autotune": (C.c_int, None),
    "afem_batch_failure_test": (C.c_int, [_P, C.c_int, C.c_longlong]),
}

_lib = None


def lib():
    """Load libafem_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: the CUDA library must be built first "
                               "(python -c 'import __graft_entry__ as g; g.build()'); there is no fallback")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            if args is not None:      # None: variadic-looking signatures declared at the call site
                fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status != AFEM_OK:
        msg = lib().afem_last_error().decode(errors="replace")
        raise AfemError(status, f"{what}: {msg}" if what else msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args), name)
