// afem_gb300.hpp -- header-only C++ mirror of ArcaneFEM's node-wise assembly
// and CSR linear-system interfaces, on top of the C ABI (afem_gb300.h).
//
//   afem::BSRFormat            femutils/BSRFormat.h:157-249 (atomic-free path):
//                              initialize / computeSparsity / assembleBilinear /
//                              toLinearSystem / matrix / resetMatrixValues
//   afem::CsrDoFLinearSystem   femutils/internal/CsrDoFLinearSystemImpl.h:36-113
//                              behind femutils/internal/IDoFLinearSystemImpl.h:37-70
//
// Errors are thrown as afem::Error (the counterpart of ARCANE_FATAL /
// ARCANE_THROW); device memory is allocated with cudaMallocAsync on the
// context's stream and released by the destructors.  The Arcane service
// (GB300LinearSystem) that plugs the library behind IDoFLinearSystemImpl is
// arcanefem_gb300/arcane/GB300DoFLinearSystem.{h,cc}.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>

#include "afem_gb300.h"

namespace afem {

class Error : public std::runtime_error {
 public:
  Error(afem_status s, const std::string& what) : std::runtime_error(what), status_(s) {}
  afem_status status() const { return status_; }

 private:
  afem_status status_;
};

inline void check(afem_status s, const char* call) {
  if (s != AFEM_OK) throw Error(s, std::string(call) + ": " + afem_last_error());
}

inline void check_cuda(cudaError_t e, const char* call) {
  if (e != cudaSuccess) throw Error(AFEM_ERR_CUDA, std::string(call) + ": " + cudaGetErrorString(e));
}

// Owning device array on a stream (stream-ordered allocation).
template <class T>
class DeviceArray {
 public:
  DeviceArray() = default;
  DeviceArray(size_t n, cudaStream_t s) : n_(n), s_(s) {
    if (n_) check_cuda(cudaMallocAsync(reinterpret_cast<void**>(&p_), n_ * sizeof(T), s_), "cudaMallocAsync");
  }
  DeviceArray(const DeviceArray&) = delete;
  DeviceArray& operator=(const DeviceArray&) = delete;
  DeviceArray(DeviceArray&& o) noexcept { swap(o); }
  DeviceArray& operator=(DeviceArray&& o) noexcept {
    swap(o);
    return *this;
  }
  ~DeviceArray() {
    if (p_) cudaFreeAsync(p_, s_);
  }
  T* data() { return p_; }
  const T* data() const { return p_; }
  size_t size() const { return n_; }
  void zero() { check_cuda(cudaMemsetAsync(p_, 0, n_ * sizeof(T), s_), "cudaMemsetAsync"); }

 private:
  void swap(DeviceArray& o) {
    std::swap(p_, o.p_);
    std::swap(n_, o.n_);
    std::swap(s_, o.s_);
  }
  T* p_ = nullptr;
  size_t n_ = 0;
  cudaStream_t s_ = nullptr;
};

// The RunQueue counterpart: a stream and the library's scratch arena.
class Context {
 public:
  explicit Context(cudaStream_t stream = nullptr) : stream_(stream) {
    check(afem_context_create(&h_, stream), "afem_context_create");
  }
  Context(const Context&) = delete;
  Context& operator=(const Context&) = delete;
  ~Context() { afem_context_destroy(h_); }
  afem_context handle() const { return h_; }
  cudaStream_t stream() const { return stream_; }
  void barrier() { check(afem_context_synchronize(h_), "afem_context_synchronize"); }

 private:
  afem_context h_ = nullptr;
  cudaStream_t stream_;
};

// A P1 mesh already in device memory (non-owning).
struct MeshView {
  int dim = 0;
  int nb_node = 0;
  int nb_cell = 0;
  const double* coords = nullptr;       // [nb_node][3]
  const int32_t* cell_nodes = nullptr;  // [nb_cell][dim+1], 16-byte aligned for tetrahedra
};

class CsrDoFLinearSystem;

// Node-wise (atomic-free) BSR assembly: BSRFormat with use_atomic_free = true.
class BSRFormat {
 public:
  BSRFormat(Context& ctx, const MeshView& mesh) : ctx_(ctx), mesh_(mesh) {}

  // BSRFormat::initialize(mesh, nb_dof, does_linear_system_use_csr, use_atomic_free)
  void initialize(int nb_dof, bool does_linear_system_use_csr, int col_order = AFEM_COLS_ASCENDING) {
    if (nb_dof != 1 && !(nb_dof == 3 && mesh_.dim == 3))
      throw Error(AFEM_ERR_BAD_ARG, "BSRFormat::initialize: nb_dof must be 1, or 3 on tetrahedra");
    nb_dof_ = nb_dof;
    per_block_ = !does_linear_system_use_csr;
    col_order_ = col_order;
    const size_t npc = mesh_.dim + 1, total = (size_t)mesh_.nb_cell * npc;
    cudaStream_t s = ctx_.stream();
    nc_ptr_ = DeviceArray<int32_t>(mesh_.nb_node + 1, s);
    nc_cell_ = DeviceArray<int32_t>(total, s);
    nc_local_ = DeviceArray<uint8_t>(total, s);
    nc_inverse_ = DeviceArray<int32_t>(total, s);
    check(afem_node_cell_build(ctx_.handle(), mesh_.nb_node, mesh_.nb_cell, (int)npc, mesh_.cell_nodes, nc_ptr_.data(),
                               nc_cell_.data(), nc_local_.data(), nc_inverse_.data()),
          "afem_node_cell_build");
  }

  // BSRFormat::computeSparsity
  void computeSparsity() {
    const int npc = mesh_.dim + 1;
    cudaStream_t s = ctx_.stream();
    row_ptr_ = DeviceArray<int32_t>(mesh_.nb_node + 1, s);
    int64_t nnzb = 0;
    check(afem_sparsity_rows(ctx_.handle(), mesh_.nb_node, npc, mesh_.cell_nodes, nc_ptr_.data(), nc_cell_.data(),
                             row_ptr_.data(), &nnzb),
          "afem_sparsity_rows");
    nnzb_ = nnzb;
    cols_ = DeviceArray<int32_t>(nnzb, s);
    nc_slot_ = DeviceArray<uint8_t>((size_t)mesh_.nb_cell * npc * npc, s);
    check(afem_sparsity_cols(ctx_.handle(), mesh_.nb_node, npc, mesh_.cell_nodes, nc_ptr_.data(), nc_cell_.data(),
                             nc_local_.data(), row_ptr_.data(), col_order_, cols_.data(), nc_slot_.data()),
          "afem_sparsity_cols");
    values_ = DeviceArray<double>((size_t)nnzb_ * nb_dof_ * nb_dof_, s);
    values_.zero();
  }

  // assembleBilinearAtomicFree with _computeElementVector{Tria3,Tetra4}Gpu
  void assemblePoisson(const double* cell_coeff = nullptr) {
    afem_mesh_view v = view();
    check(afem_assemble_poisson_p1(ctx_.handle(), &v, row_ptr_.data(), cell_coeff, values_.data()),
          "afem_assemble_poisson_p1");
  }

  // assembleBilinearAtomicFree with computeElementVectorTetra4Gpu (elasticity)
  void assembleElasticity(double lambda, double mu) {
    afem_mesh_view v = view();
    check(afem_assemble_elasticity_tet4(ctx_.handle(), &v, row_ptr_.data(), lambda, mu,
                                        per_block_ ? AFEM_LAYOUT_PER_BLOCK : AFEM_LAYOUT_PER_ROW, values_.data()),
          "afem_assemble_elasticity_tet4");
  }

  void resetMatrixValues() { values_.zero(); }

  // BSRFormat::toLinearSystem, CSR path (BSRMatrix::toCsr done on the device)
  void toLinearSystem(CsrDoFLinearSystem& ls);

  void applyConstantSourceToRhs(double qdot, double* rhs) {
    afem_mesh_view v = view();
    check(afem_rhs_constant_source(ctx_.handle(), &v, qdot, nb_dof_, rhs), "afem_rhs_constant_source");
  }

  afem_mesh_view view() const {
    afem_mesh_view v{};
    v.dim = mesh_.dim;
    v.nb_node = mesh_.nb_node;
    v.nb_cell = mesh_.nb_cell;
    v.coords_d = mesh_.coords;
    v.cell_nodes_d = mesh_.cell_nodes;
    v.nc_ptr_d = nc_ptr_.data();
    v.nc_cell_d = nc_cell_.data();
    v.nc_local_d = nc_local_.data();
    v.nc_slot_d = nc_slot_.data();
    v.nc_inverse_d = nc_inverse_.data();
    return v;
  }

  int nbDof() const { return nb_dof_; }
  int64_t nbNonZeroBlocks() const { return nnzb_; }
  const int32_t* rowIndex() const { return row_ptr_.data(); }
  const int32_t* columns() const { return cols_.data(); }
  double* values() { return values_.data(); }

 private:
  Context& ctx_;
  MeshView mesh_;
  int nb_dof_ = 1;
  bool per_block_ = false;
  int col_order_ = AFEM_COLS_ASCENDING;
  int64_t nnzb_ = 0;
  DeviceArray<int32_t> nc_ptr_, nc_cell_, nc_inverse_, row_ptr_, cols_, csr_row_ptr_, csr_cols_;
  DeviceArray<uint8_t> nc_local_, nc_slot_;
  DeviceArray<double> values_;
};

// CsrDoFLinearSystemImpl over the device CSR view.
class CsrDoFLinearSystem {
 public:
  CsrDoFLinearSystem(Context& ctx, int nb_dof) : ctx_(ctx) {
    check(afem_ls_create(ctx.handle(), nb_dof, &h_), "afem_ls_create");
    check(afem_ls_dof_variables(h_, &rhs_, &sol_, &fi_, &fv_, &ei_, &ev_), "afem_ls_dof_variables");
  }
  CsrDoFLinearSystem(const CsrDoFLinearSystem&) = delete;
  CsrDoFLinearSystem& operator=(const CsrDoFLinearSystem&) = delete;
  ~CsrDoFLinearSystem() { afem_ls_destroy(h_); }

  bool hasSetCSRValues() const { return true; }
  void setCSRValues(const int32_t* row_ptr, const int32_t* cols, double* values, int64_t nnz) {
    check(afem_ls_set_csr_values(h_, row_ptr, cols, values, nnz), "afem_ls_set_csr_values");
  }
  void matrixAddValue(int32_t row, int32_t col, double v) {
    check(afem_ls_matrix_add_value(h_, row, col, v), "afem_ls_matrix_add_value");
  }
  void matrixSetValue(int32_t row, int32_t col, double v) {
    check(afem_ls_matrix_set_value(h_, row, col, v), "afem_ls_matrix_set_value");
  }
  void eliminateRow(int32_t row, double v) { check(afem_ls_eliminate_row(h_, row, v), "eliminateRow"); }
  void eliminateRowColumn(int32_t row, double v) {
    check(afem_ls_eliminate_row_column(h_, row, v), "eliminateRowColumn");
  }
  void clearValues() { check(afem_ls_clear_values(h_), "afem_ls_clear_values"); }
  void applyMatrixTransformation() {
    check(afem_ls_apply_matrix_transformation(h_), "afem_ls_apply_matrix_transformation");
  }
  void applyRHSTransformation() { check(afem_ls_apply_rhs_transformation(h_), "afem_ls_apply_rhs_transformation"); }
  afem_solve_info solve(const afem_solver_options* opt = nullptr) {
    afem_solve_info info{};
    check(afem_ls_solve(h_, opt, &info), "afem_ls_solve");
    return info;
  }
  // Gpu::BoundaryConditions helpers (femutils/ArcaneFemFunctionsGpu.cc:54-105)
  void applyDirichletViaPenalty(const int32_t* nodes, int nb, int nb_dof_per_node, int dof, double value,
                                double penalty = 1e30) {
    check(afem_dirichlet_penalty(h_, nb, nodes, nb_dof_per_node, dof, value, penalty), "afem_dirichlet_penalty");
  }
  void applyDirichletViaElimination(int type, const int32_t* nodes, int nb, int nb_dof_per_node, int dof,
                                    double value) {
    check(afem_dirichlet_elimination(h_, type, nb, nodes, nb_dof_per_node, dof, value), "afem_dirichlet_elimination");
  }
  double* rhsVariable() { return rhs_; }
  double* solutionVariable() { return sol_; }
  uint8_t* getForcedInfo() { return fi_; }
  double* getForcedValue() { return fv_; }
  uint8_t* getEliminationInfo() { return ei_; }
  double* getEliminationValue() { return ev_; }

 private:
  Context& ctx_;
  afem_linear_system h_ = nullptr;
  double *rhs_ = nullptr, *sol_ = nullptr, *fv_ = nullptr, *ev_ = nullptr;
  uint8_t *fi_ = nullptr, *ei_ = nullptr;
};

inline void BSRFormat::toLinearSystem(CsrDoFLinearSystem& ls) {
  if (nb_dof_ == 1) {
    ls.setCSRValues(row_ptr_.data(), cols_.data(), values_.data(), nnzb_);
    return;
  }
  if (per_block_)
    throw Error(AFEM_ERR_BAD_ARG, "BSRFormat::toLinearSystem: the CSR path needs the per-row value layout");
  cudaStream_t s = ctx_.stream();
  const int b = nb_dof_;
  csr_row_ptr_ = DeviceArray<int32_t>((size_t)mesh_.nb_node * b + 1, s);
  csr_cols_ = DeviceArray<int32_t>((size_t)nnzb_ * b * b, s);
  check(afem_bsr_to_csr_structure(ctx_.handle(), mesh_.nb_node, b, row_ptr_.data(), cols_.data(), csr_row_ptr_.data(),
                                  csr_cols_.data()),
        "afem_bsr_to_csr_structure");
  ls.setCSRValues(csr_row_ptr_.data(), csr_cols_.data(), values_.data(), nnzb_ * b * b);
}

}  // namespace afem
