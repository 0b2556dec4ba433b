// Linear-system handle mirroring CsrDoFLinearSystemImpl
// (femutils/internal/CsrDoFLinearSystemImpl.h:36-113,
//  femutils/CsrDoFLinearSystemImpl.cc, femutils/DoFLinearSystemImplBase.cc):
// DoF variables on the device, a non-owning CSR view, Dirichlet flagging and
// the matrix / right-hand-side transformations.  The reference keeps the
// row-column elimination bookkeeping on the host (an ordered std::map filled
// by a host loop over all nonzeros, CsrDoFLinearSystemImpl.cc:187-230, then
// DoFLinearSystemImplBase.cc:55-88); here a device copy of the
// pre-elimination values plays the map's role and the rhs correction is a
// row-parallel kernel that subtracts in the same (increasing row) order.
#include "afem_internal.cuh"

struct afem_linear_system_s {
  afem_context ctx = nullptr;
  int n = 0;
  double* rhs = nullptr;
  double* sol = nullptr;
  uint8_t* forced_info = nullptr;
  double* forced_value = nullptr;
  uint8_t* elim_info = nullptr;
  double* elim_value = nullptr;
  // non-owning CSR view
  const int32_t* row_ptr = nullptr;
  const int32_t* cols = nullptr;
  double* values = nullptr;
  int64_t nnz = 0;
  // row offsets [n + 1] owned by the system when the matrix came as a
  // reference CSR view (afem_ls_set_csr_view); 1 if that view has unused slots
  int32_t* view_row_ptr = nullptr;
  int padded = 0;
  // the learned preconditioner (precond = AFEM_PRECOND_LEARNED) and the
  // version of the matrix values its operator was last set from
  afem_mpnn learned = nullptr;
  int64_t values_version = 1;
  int64_t learned_version = 0;
  // row-column elimination bookkeeping
  int has_rc = 0;
  double* rc_saved = nullptr;
  int64_t rc_cap = 0;
  int* flag = nullptr;
};

namespace afem {

__global__ void k_penalty(int nb_sel, const int32_t* __restrict__ nodes, int nb_dof, int dof_index, double value,
                          double penalty, int n, uint8_t* __restrict__ fi, double* __restrict__ fv,
                          double* __restrict__ rhs, int* __restrict__ err) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nb_sel; s += gridDim.x * blockDim.x) {
    int64_t d = (int64_t)nodes[s] * nb_dof + dof_index;
    if (d < 0 || d >= n) {
      atomicOr(err, 1);
      continue;
    }
    fi[d] = 1;
    fv[d] = penalty;
    rhs[d] = penalty * value;
  }
}

__global__ void k_elim_flag(int nb_sel, const int32_t* __restrict__ nodes, int nb_dof, int dof_index, double value,
                            uint8_t type, int n, uint8_t* __restrict__ ei, double* __restrict__ ev,
                            int* __restrict__ err) {
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nb_sel; s += gridDim.x * blockDim.x) {
    int64_t d = (int64_t)nodes[s] * nb_dof + dof_index;
    if (d < 0 || d >= n) {
      atomicOr(err, 1);
      continue;
    }
    ei[d] = type;
    ev[d] = value;
  }
}

__global__ void k_any_rc(int n, const uint8_t* __restrict__ ei, int* __restrict__ flag) {
  int found = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    found |= (ei[i] == AFEM_ELIMINATE_ROW_COLUMN);
  if (__syncthreads_or(found) && threadIdx.x == 0) atomicOr(flag, 1);
}

// Row elimination (CsrDoFLinearSystemImpl.cc:126-152), row-column
// elimination with its column_index > 0 test (:88-121) and forced diagonal
// values (:50-72), fused per row: each step only reads flags and writes the
// row's own entries, so the order of the reference's three kernels is kept.
__global__ void k_transform(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                            double* __restrict__ vals, const uint8_t* __restrict__ fi, const double* __restrict__ fv,
                            const uint8_t* __restrict__ ei, int has_rc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t b = rp[i], e = rp[i + 1];
    const uint8_t ri = ei[i];
    if (ri == AFEM_ELIMINATE_ROW)
      for (int32_t k = b; k < e; ++k) vals[k] = (cols[k] == i) ? 1.0 : 0.0;
    if (has_rc) {
      const bool is_row = ri == AFEM_ELIMINATE_ROW || ri == AFEM_ELIMINATE_ROW_COLUMN;
      for (int32_t k = b; k < e; ++k) {
        const int32_t c = cols[k];
        if (c > 0) {
          const uint8_t ci = ei[c];
          const bool is_col = ci == AFEM_ELIMINATE_ROW || ci == AFEM_ELIMINATE_ROW_COLUMN;
          if (is_row || is_col) vals[k] = (c == i) ? 1.0 : 0.0;
        }
      }
    }
    if (fi[i]) {
      for (int32_t k = b; k < e; ++k)
        if (cols[k] == i) {
          vals[k] = fv[i];
          break;
        }
    }
  }
}

// The pre-elimination values of the row-column eliminated rows (the only
// ones k_rc_rhs reads), at their own positions of `saved`.
__global__ void k_save_rc_rows(int n, const int32_t* __restrict__ rp, const double* __restrict__ vals,
                               const uint8_t* __restrict__ ei, double* __restrict__ saved) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (ei[i] != AFEM_ELIMINATE_ROW_COLUMN) continue;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) saved[k] = vals[k];
  }
}

// rhs_j -= A_ij g_i for stored (i, j), i != j, i row-column eliminated, in
// increasing i (DoFLinearSystemImplBase.cc:55-88); unfused multiply and
// subtract as the reference's host code.  A_ij is read from the saved
// pre-elimination values of row i.
__global__ void k_rc_rhs(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                         const double* __restrict__ saved, const uint8_t* __restrict__ ei,
                         const double* __restrict__ ev, double* __restrict__ rhs) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double v = rhs[j];
    bool touched = false;
    for (int32_t k = rp[j]; k < rp[j + 1]; ++k) {
      const int32_t i = cols[k];
      if (i < 0 || i == j || ei[i] != AFEM_ELIMINATE_ROW_COLUMN) continue;
      for (int32_t q = rp[i]; q < rp[i + 1]; ++q)
        if (cols[q] == j) {
          v = __dsub_rn(v, __dmul_rn(saved[q], ev[i]));
          touched = true;
          break;
        }
    }
    if (touched) rhs[j] = v;
  }
}

// rhs_i = g_i on eliminated rows (CsrDoFLinearSystemImpl.cc:157-182).
__global__ void k_rhs_elim(int n, const uint8_t* __restrict__ ei, const double* __restrict__ ev,
                           double* __restrict__ rhs) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint8_t t = ei[i];
    if (t == AFEM_ELIMINATE_ROW || t == AFEM_ELIMINATE_ROW_COLUMN) rhs[i] = ev[i];
  }
}

// matrixAddValue / matrixSetValue on one entry (linear search in the row).
__global__ void k_entry(const int32_t* __restrict__ rp, const int32_t* __restrict__ cols, double* __restrict__ vals,
                        int32_t row, int32_t col, double value, int add, int* __restrict__ flag) {
  for (int32_t k = rp[row]; k < rp[row + 1]; ++k)
    if (cols[k] == col) {
      vals[k] = add ? vals[k] + value : value;
      return;
    }
  *flag = 1;
}

// Row offsets of a reference CSR view (rows without the trailing entry, the
// last row ending at nb_column) and its checks: flags bit 0 = a bad row start
// or count, bit 1 = a column out of range, bit 2 = a slot past a row's count
// that is not -1, bit 3 = the view has unused (-1) slots.
__global__ void k_view_rows(int n, const int32_t* __restrict__ rows, const int32_t* __restrict__ nb_col,
                            int64_t nb_column, const int32_t* __restrict__ cols, int32_t* __restrict__ rp,
                            int* __restrict__ flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
    if (i == n) {
      rp[n] = (int32_t)nb_column;
      continue;
    }
    const int32_t b = rows[i];
    const int64_t e = i + 1 < n ? (int64_t)rows[i + 1] : nb_column;
    rp[i] = b;
    if (b < 0 || (int64_t)b > e) {
      atomicOr(flags, 1);
      continue;
    }
    const int64_t used = nb_col ? (int64_t)nb_col[i] : e - b;
    if (used < 0 || b + used > e) {
      atomicOr(flags, 1);
      continue;
    }
    int f = 0;
    for (int64_t k = b; k < e; ++k) {
      const int32_t c = cols[k];
      if (c >= n) f |= 2;
      if (c < -1) f |= 2;
      if (c == -1) f |= 8;
      if (k >= b + used && c != -1) f |= 4;
    }
    if (f) atomicOr(flags, f);
  }
}

afem_status solve_csr(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals,
                      const double* b, double* x, const uint8_t* forced, const afem_solver_options* opt,
                      afem_solve_info* info);

static afem_status need_view(afem_linear_system ls, const char* who) {
  AFEM_CHECK_ARG(ls != nullptr, "%s: null linear system", who);
  if (!ls->row_ptr || !ls->cols || !ls->values)
    return fail(AFEM_ERR_BAD_ARG, "%s: no CSR values set (call afem_ls_set_csr_values first)", who);
  return AFEM_OK;
}

}  // namespace afem

using namespace afem;

extern "C" {

afem_status afem_ls_create(afem_context ctx, int nb_dof, afem_linear_system* out) {
  AFEM_CHECK_ARG(ctx && out && nb_dof > 0, "afem_ls_create: bad arguments");
  *out = nullptr;
  auto* ls = new (std::nothrow) afem_linear_system_s();
  if (!ls) return fail(AFEM_ERR_OOM, "afem_ls_create: host allocation failed");
  ls->ctx = ctx;
  ls->n = nb_dof;
  const size_t n = nb_dof;
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaMallocAsync((void**)&ls->rhs, n * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&ls->sol, n * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&ls->forced_value, n * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&ls->elim_value, n * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&ls->forced_info, n, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&ls->elim_info, n, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&ls->flag, sizeof(int), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ls->rhs, 0, n * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ls->sol, 0, n * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ls->forced_value, 0, n * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ls->elim_value, 0, n * sizeof(double), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ls->forced_info, 0, n, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(ls->elim_info, 0, n, s);
  if (e != cudaSuccess) {
    afem_ls_destroy(ls);
    return cuda_fail(e, "afem_ls_create", __FILE__, __LINE__);
  }
  *out = ls;
  return AFEM_OK;
}

afem_status afem_ls_destroy(afem_linear_system ls) {
  if (!ls) return AFEM_OK;
  cudaStream_t s = ls->ctx->stream;
  void* ptrs[] = {ls->rhs, ls->sol, ls->forced_value, ls->elim_value, ls->forced_info, ls->elim_info, ls->flag,
                  ls->rc_saved, ls->view_row_ptr};
  for (void* p : ptrs)
    if (p) cudaFreeAsync(p, s);
  cudaStreamSynchronize(s);
  delete ls;
  return AFEM_OK;
}

afem_status afem_ls_set_csr_values(afem_linear_system ls, const int32_t* row_ptr_d, const int32_t* cols_d,
                                   double* values_d, int64_t nnz) {
  AFEM_CHECK_ARG(ls && row_ptr_d && cols_d && values_d && nnz > 0, "afem_ls_set_csr_values: bad arguments");
  ++ls->values_version;
  ls->row_ptr = row_ptr_d;
  ls->cols = cols_d;
  ls->values = values_d;
  ls->nnz = nnz;
  ls->padded = 0;
  return AFEM_OK;
}

afem_status afem_ls_set_csr_view(afem_linear_system ls, int32_t nb_row, const int32_t* rows_d,
                                 const int32_t* rows_nb_column_d, int64_t nb_column, const int32_t* columns_d,
                                 double* values_d) {
  AFEM_CHECK_ARG(ls && rows_d && columns_d && values_d && nb_column > 0 && nb_column <= INT32_MAX,
                 "afem_ls_set_csr_view: bad arguments");
  AFEM_CHECK_ARG(nb_row == ls->n, "afem_ls_set_csr_view: %d rows for a system of %d DoFs (the DoF family must be "
                                  "compacted, one row per DoF)", nb_row, ls->n);
  afem_context ctx = ls->ctx;
  if (!ls->view_row_ptr)
    AFEM_CUDA(cudaMallocAsync((void**)&ls->view_row_ptr, sizeof(int32_t) * ((size_t)ls->n + 1), ctx->stream));
  AFEM_CUDA(cudaMemsetAsync(ls->flag, 0, sizeof(int), ctx->stream));
  AFEM_TRY(launch(ctx, k_view_rows, grid_for(ctx, (int64_t)ls->n + 1, 256), 256, 0, ls->n, rows_d, rows_nb_column_d,
                  nb_column, columns_d, ls->view_row_ptr, ls->flag));
  int f = 0;
  AFEM_TRY(read_scalar(ctx, ls->flag, &f));
  if (f & 1)
    return fail(AFEM_ERR_BAD_ARG, "afem_ls_set_csr_view: a row start is negative, decreasing or past nb_column, or "
                                  "a row's column count overruns its range");
  if (f & 2) return fail(AFEM_ERR_BAD_ARG, "afem_ls_set_csr_view: a column index is below -1 or not a DoF");
  if (f & 4)
    return fail(AFEM_ERR_BAD_ARG, "afem_ls_set_csr_view: a slot past a row's column count holds a column (not -1)");
  ++ls->values_version;
  ls->row_ptr = ls->view_row_ptr;
  ls->cols = columns_d;
  ls->values = values_d;
  ls->nnz = nb_column;
  ls->padded = (f & 8) ? 1 : 0;
  return AFEM_OK;
}

afem_status afem_ls_get_csr_values(afem_linear_system ls, const int32_t** row_ptr_d, const int32_t** cols_d,
                                   double** values_d, int64_t* nnz) {
  AFEM_CHECK_ARG(ls, "afem_ls_get_csr_values: null linear system");
  if (row_ptr_d) *row_ptr_d = ls->row_ptr;
  if (cols_d) *cols_d = ls->cols;
  if (values_d) *values_d = ls->values;
  if (nnz) *nnz = ls->nnz;
  return AFEM_OK;
}

afem_status afem_ls_dof_variables(afem_linear_system ls, double** rhs, double** sol, uint8_t** fi, double** fv,
                                  uint8_t** ei, double** ev) {
  AFEM_CHECK_ARG(ls, "afem_ls_dof_variables: null linear system");
  if (rhs) *rhs = ls->rhs;
  if (sol) *sol = ls->sol;
  if (fi) *fi = ls->forced_info;
  if (fv) *fv = ls->forced_value;
  if (ei) *ei = ls->elim_info;
  if (ev) *ev = ls->elim_value;
  return AFEM_OK;
}

afem_status afem_ls_clear_values(afem_linear_system ls) {
  AFEM_CHECK_ARG(ls, "afem_ls_clear_values: null linear system");
  cudaStream_t s = ls->ctx->stream;
  AFEM_CUDA(cudaMemsetAsync(ls->forced_info, 0, ls->n, s));
  AFEM_CUDA(cudaMemsetAsync(ls->elim_info, 0, ls->n, s));
  AFEM_CUDA(cudaMemsetAsync(ls->elim_value, 0, ls->n * sizeof(double), s));
  ls->row_ptr = nullptr;
  ls->cols = nullptr;
  ls->values = nullptr;
  ls->nnz = 0;
  ls->padded = 0;
  ls->has_rc = 0;
  return AFEM_OK;
}

static afem_status entry(afem_linear_system ls, int32_t row, int32_t col, double value, int add, const char* who) {
  AFEM_TRY(need_view(ls, who));
  ++ls->values_version;
  AFEM_CHECK_ARG(row >= 0 && row < ls->n && col >= 0 && col < ls->n, "%s: (%d, %d) out of range", who, row, col);
  afem_context ctx = ls->ctx;
  AFEM_CUDA(cudaMemsetAsync(ls->flag, 0, sizeof(int), ctx->stream));
  AFEM_TRY(launch(ctx, k_entry, 1, 1, 0, ls->row_ptr, ls->cols, ls->values, row, col, value, add, ls->flag));
  int f = 0;
  AFEM_TRY(read_scalar(ctx, ls->flag, &f));
  if (f) return fail(AFEM_ERR_NOT_FOUND, "%s: entry (%d, %d) is not in the sparsity", who, row, col);
  return AFEM_OK;
}

afem_status afem_ls_matrix_add_value(afem_linear_system ls, int32_t row, int32_t col, double value) {
  return entry(ls, row, col, value, 1, "afem_ls_matrix_add_value");
}

afem_status afem_ls_matrix_set_value(afem_linear_system ls, int32_t row, int32_t col, double value) {
  return entry(ls, row, col, value, 0, "afem_ls_matrix_set_value");
}

afem_status afem_ls_eliminate_row(afem_linear_system ls, int32_t, double) {
  AFEM_CHECK_ARG(ls, "afem_ls_eliminate_row: null linear system");
  return fail(AFEM_ERR_NOT_IMPLEMENTED,
              "afem_ls_eliminate_row: not implemented on the CSR system; flag rows with afem_dirichlet_elimination");
}

afem_status afem_ls_eliminate_row_column(afem_linear_system ls, int32_t, double) {
  AFEM_CHECK_ARG(ls, "afem_ls_eliminate_row_column: null linear system");
  return fail(AFEM_ERR_NOT_IMPLEMENTED,
              "afem_ls_eliminate_row_column: not implemented on the CSR system; flag rows with "
              "afem_dirichlet_elimination");
}

afem_status afem_dirichlet_penalty(afem_linear_system ls, int nb_sel, const int32_t* nodes_d, int nb_dof_per_node,
                                   int dof_index, double value, double penalty) {
  AFEM_CHECK_ARG(ls && nb_sel >= 0 && nb_dof_per_node >= 1 && dof_index >= 0 && dof_index < nb_dof_per_node,
                 "afem_dirichlet_penalty: bad arguments");
  if (nb_sel == 0) return AFEM_OK;
  AFEM_CHECK_ARG(nodes_d, "afem_dirichlet_penalty: null node list");
  afem_context ctx = ls->ctx;
  AFEM_CUDA(cudaMemsetAsync(ls->flag, 0, sizeof(int), ctx->stream));
  AFEM_TRY(launch(ctx, k_penalty, grid_for(ctx, nb_sel, 256), 256, 0, nb_sel, nodes_d, nb_dof_per_node, dof_index,
                  value, penalty, ls->n, ls->forced_info, ls->forced_value, ls->rhs, ls->flag));
  int f = 0;
  AFEM_TRY(read_scalar(ctx, ls->flag, &f));
  if (f) return fail(AFEM_ERR_BAD_ARG, "afem_dirichlet_penalty: node id out of range");
  return AFEM_OK;
}

afem_status afem_dirichlet_elimination(afem_linear_system ls, int type, int nb_sel, const int32_t* nodes_d,
                                       int nb_dof_per_node, int dof_index, double value) {
  AFEM_CHECK_ARG(ls && nb_sel >= 0 && nb_dof_per_node >= 1 && dof_index >= 0 && dof_index < nb_dof_per_node,
                 "afem_dirichlet_elimination: bad arguments");
  AFEM_CHECK_ARG(type == AFEM_ELIMINATE_ROW || type == AFEM_ELIMINATE_ROW_COLUMN,
                 "afem_dirichlet_elimination: bad elimination type %d", type);
  if (nb_sel == 0) return AFEM_OK;
  AFEM_CHECK_ARG(nodes_d, "afem_dirichlet_elimination: null node list");
  afem_context ctx = ls->ctx;
  AFEM_CUDA(cudaMemsetAsync(ls->flag, 0, sizeof(int), ctx->stream));
  AFEM_TRY(launch(ctx, k_elim_flag, grid_for(ctx, nb_sel, 256), 256, 0, nb_sel, nodes_d, nb_dof_per_node, dof_index,
                  value, (uint8_t)type, ls->n, ls->elim_info, ls->elim_value, ls->flag));
  int f = 0;
  AFEM_TRY(read_scalar(ctx, ls->flag, &f));
  if (f) return fail(AFEM_ERR_BAD_ARG, "afem_dirichlet_elimination: node id out of range");
  return AFEM_OK;
}

afem_status afem_ls_apply_matrix_transformation(afem_linear_system ls) {
  AFEM_TRY(need_view(ls, "afem_ls_apply_matrix_transformation"));
  ++ls->values_version;
  afem_context ctx = ls->ctx;
  // _fillRowColumnEliminationInfos: is any DoF RowColumn-eliminated?
  AFEM_CUDA(cudaMemsetAsync(ls->flag, 0, sizeof(int), ctx->stream));
  AFEM_TRY(launch(ctx, k_any_rc, grid_for(ctx, ls->n, 256), 256, 0, ls->n, (const uint8_t*)ls->elim_info, ls->flag));
  AFEM_TRY(read_scalar(ctx, ls->flag, &ls->has_rc));
  if (ls->has_rc) {
    if (ls->rc_cap < ls->nnz) {
      if (ls->rc_saved) AFEM_CUDA(cudaFreeAsync(ls->rc_saved, ctx->stream));
      ls->rc_saved = nullptr;
      ls->rc_cap = 0;
      AFEM_CUDA(cudaMallocAsync((void**)&ls->rc_saved, sizeof(double) * ls->nnz, ctx->stream));
      ls->rc_cap = ls->nnz;
    }
    AFEM_TRY(launch(ctx, k_save_rc_rows, grid_for(ctx, ls->n, 256), 256, 0, ls->n, ls->row_ptr,
                    (const double*)ls->values, (const uint8_t*)ls->elim_info, ls->rc_saved));
  }
  return launch(ctx, k_transform, grid_for(ctx, ls->n, 256), 256, 0, ls->n, ls->row_ptr, ls->cols, ls->values,
                (const uint8_t*)ls->forced_info, (const double*)ls->forced_value, (const uint8_t*)ls->elim_info,
                ls->has_rc);
}

afem_status afem_ls_apply_rhs_transformation(afem_linear_system ls) {
  AFEM_TRY(need_view(ls, "afem_ls_apply_rhs_transformation"));
  afem_context ctx = ls->ctx;
  if (ls->has_rc)
    AFEM_TRY(launch(ctx, k_rc_rhs, grid_for(ctx, ls->n, 256), 256, 0, ls->n, ls->row_ptr, ls->cols,
                    (const double*)ls->rc_saved, (const uint8_t*)ls->elim_info, (const double*)ls->elim_value,
                    ls->rhs));
  return launch(ctx, k_rhs_elim, grid_for(ctx, ls->n, 256), 256, 0, ls->n, (const uint8_t*)ls->elim_info,
                (const double*)ls->elim_value, ls->rhs);
}

afem_status afem_ls_set_learned_preconditioner(afem_linear_system ls, afem_mpnn net) {
  AFEM_CHECK_ARG(ls, "afem_ls_set_learned_preconditioner: null linear system");
  ls->learned = net;
  ls->learned_version = 0;
  return AFEM_OK;
}

afem_status afem_ls_solve(afem_linear_system ls, const afem_solver_options* opt, afem_solve_info* info) {
  AFEM_TRY(need_view(ls, "afem_ls_solve"));
  if (opt && opt->precond == AFEM_PRECOND_LEARNED) {
    if (!ls->learned)
      return fail(AFEM_ERR_BAD_ARG, "afem_ls_solve: precond = learned needs a network "
                                    "(afem_ls_set_learned_preconditioner)");
    if (ls->padded)
      return fail(AFEM_ERR_NOT_IMPLEMENTED, "afem_ls_solve: the learned preconditioner needs a CSR view without "
                                            "unused slots");
    if (ls->learned_version != ls->values_version) {   // the matrix changed: new Galerkin values and weights
      AFEM_TRY(afem_mpnn_set_operator(ls->learned, ls->n, ls->row_ptr, ls->cols, ls->values));
      ls->learned_version = ls->values_version;
    }
    return fcg_solve(ls->ctx, ls->n, ls->row_ptr, ls->cols, ls->values, ls->rhs, ls->sol,
                     opt->skip_forced_rows ? ls->forced_info : nullptr, ls->learned, opt, info);
  }
  return solve_csr(ls->ctx, ls->n, ls->row_ptr, ls->cols, ls->values, ls->rhs, ls->sol, ls->forced_info, opt, info);
}

}  // extern "C"
