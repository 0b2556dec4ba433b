/*
 * afem_oracle.h -- CPU restatement of ArcaneFEM's node-wise P1 assembly path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * implementation in arcanefem_gb300/.  Only tests/, __graft_entry__.smoke()
 * and the cpu_baseline / --impl reference legs of bench.py may load it.  The
 * product path never calls it and has no CPU fallback.
 *
 * Every function restates the reference arithmetic in the reference's own
 * operation order (no FMA contraction: built with -ffp-contract=off), citing
 * the reference file:line it follows.  Paths are relative to the arcanefem
 * source tree.
 *
 * Conventions shared with the CUDA library:
 *   coords      : double[nb_node][3]   (Real3 AoS, z = 0 in 2D)
 *   cell_nodes  : int32[nb_cell][npc]  (npc = 3 triangles, 4 tetrahedra)
 *   row_ptr     : int32[nb_row + 1]
 *   DoF numbering: dof = node * nb_dof + component (FemDoFsOnNodes.cc:72-112)
 */
#ifndef AFEM_ORACLE_H
#define AFEM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* element kinds */
enum {
  AFO_POISSON_TRI3 = 0,       /* modules/poisson/ElementMatrix.h:54-63 */
  AFO_POISSON_TET4 = 1,       /* modules/poisson/ElementMatrix.h:107-118 */
  AFO_ELASTICITY_TET4 = 2,    /* modules/elasticity/ElementMatrix.h:216-301 */
  AFO_TESTLAB_TRI3 = 3,       /* modules/testlab/FemModule.h:471-495 + NodeWiseCsrBiliAssembly.cc:194-211 */
  AFO_TESTLAB_TET4 = 4,       /* modules/testlab/FemModule.h:499-538 + NodeWiseCsrBiliAssembly.cc:269-290 */
  AFO_POISSON_QUAD4 = 5,      /* modules/poisson/ElementMatrixHexQuad.h:63-91 */
  AFO_POISSON_HEXA8 = 6       /* modules/poisson/ElementMatrixHexQuad.h:239-266 */
};

/* node -> cell adjacency, cells ascending per node, plus the local index of
 * the node inside each incident cell.  Returns 0, or -1 on a bad node id. */
int afo_node_cell(int nb_node, int nb_cell, int npc, const int32_t* cell_nodes,
                  int32_t* nc_ptr, int32_t* nc_cell, uint8_t* nc_local);

/* Sparsity by edge pack / sort / unique / count / scan
 * (femutils/BSRFormat.cc:799-1006).  Rows are node rows (block rows).
 * Columns come out in canonical order: ascending (self_last = 0) or the
 * neighbours ascending followed by the diagonal (self_last = 1, the
 * atomic-free convention of BSRFormat.cc:658-672,758-770).
 * Returns the number of column entries, or -1 if cap is too small. */
int64_t afo_sparsity(int nb_node, int nb_cell, int npc, const int32_t* cell_nodes, int self_last,
                     int32_t* row_ptr, int32_t* cols, int64_t cap);

/* Element row vectors of the reference element kernels. */
void afo_elem_vec_poisson_tri3(const double* coords, const int32_t* cn, int local, double out[3]);
void afo_elem_vec_poisson_tet4(const double* coords, const int32_t* cn, int local, double out[4]);
void afo_elem_vec_testlab_tri3(const double* coords, const int32_t* cn, int local, double out[3]);
void afo_elem_vec_testlab_tet4(const double* coords, const int32_t* cn, int local, double out[4]);
void afo_elem_vec_elasticity_tet4(const double* coords, const int32_t* cn, double lambda, double mu,
                                  int local, double out[36]);

/* Node-wise (atomic-free) assembly: BSRFormat.h:406-470 (per-block value
 * layout) and BSRFormat.h:473-537 (per-row, CSR-compatible layout);
 * NodeWiseCsrBiliAssembly.cc:157-297 for the testlab kinds.
 * values must be zeroed by the caller (BSRMatrix::initialize fills 0).
 * cell_coeff (may be NULL) multiplies each element contribution.
 * nb_threads > 1 splits the node loop over that many OpenMP threads. */
int afo_assemble_nodewise(int kind, int nb_node, int nb_cell, const double* coords, const int32_t* cell_nodes,
                          const int32_t* nc_ptr, const int32_t* nc_cell, const int32_t* row_ptr,
                          const int32_t* cols, int per_block_layout, double lambda, double mu,
                          const double* cell_coeff, double* values, int nb_threads);

/* Constant source: rhs[dof(node, 0)] = sum_cells qdot * measure / nb_node_of_cell
 * (femutils/ArcaneFemFunctionsGpu.h:676-708). */
void afo_rhs_constant_source(int dim, int nb_node, const double* coords, const int32_t* cell_nodes, int npc,
                             const int32_t* nc_ptr, const int32_t* nc_cell, double qdot, int nb_dof,
                             double* rhs);

/* Body force on tetrahedra, cell loop with += (modules/elasticity/BodyForce.h:148-160). */
void afo_rhs_constant_source_q1(int dim, int nb_node, const double* coords, const int32_t* cell_nodes,
                                const int32_t* nc_ptr, const int32_t* nc_cell, double qdot, int nb_dof,
                                double* rhs);
void afo_rhs_body_force_tet4(int nb_cell, const double* coords, const int32_t* cell_nodes, const double f[3],
                             double* rhs);
void afo_rhs_boundary_faces(int dim, int nb_face, const double* coords, const int32_t* face_nodes,
                            const uint8_t* outward, int mode, const double g[3], int nb_dof, double* rhs);

/* Penalty flagging (femutils/ArcaneFemFunctionsGpu.cc:54-78). */
void afo_dirichlet_penalty(int nb_sel, const int32_t* nodes, int nb_dof, int dof_index, double value,
                           double penalty, uint8_t* forced_info, double* forced_value, double* rhs);
/* Row / row-column elimination flagging (ArcaneFemFunctionsGpu.cc:83-105). */
void afo_dirichlet_elimination(int nb_sel, const int32_t* nodes, int nb_dof, int dof_index, double value,
                               uint8_t elimination_type, uint8_t* elim_info, double* elim_value);

/* CsrDoFLinearSystemImpl::applyMatrixTransformation (CsrDoFLinearSystemImpl.cc:235-242).
 * rc_saved (nnz doubles, may be NULL when no RowColumn flag is set) receives the
 * pre-elimination values that _fillRowColumnEliminationInfos keeps (:187-230);
 * rc_mask (nnz bytes) marks which entries were kept. */
void afo_apply_matrix_transformation(int nb_row, const int32_t* row_ptr, const int32_t* cols, double* values,
                                     const uint8_t* forced_info, const double* forced_value,
                                     const uint8_t* elim_info, const double* elim_value,
                                     double* rc_saved, uint8_t* rc_mask);
/* CsrDoFLinearSystemImpl::applyRHSTransformation (CsrDoFLinearSystemImpl.cc:247-253,
 * DoFLinearSystemImplBase.cc:55-88). */
void afo_apply_rhs_transformation(int nb_row, const int32_t* row_ptr, const int32_t* cols,
                                  const uint8_t* elim_info, const double* elim_value,
                                  const double* rc_saved, const uint8_t* rc_mask, double* rhs);

/* y = A x (CSR, FP64). */
void afo_spmv(int nb_row, const int32_t* row_ptr, const int32_t* cols, const double* values, const double* x,
              double* y);

/* Diagonal (Jacobi) preconditioned CG, relative two-norm stop ||r|| <= rtol ||b||
 * (femutils/DoFLinearSystem.cc:151-159 diagonal PCG; HypreDoFLinearSystem.cc:596-603 stop).
 * norm_skip (may be NULL): rows flagged 1 are left out of both norms of the
 * stopping test, so that penalty rows (P g with P = 1e30) do not swamp it.
 * Returns iterations used (negative on breakdown); *relres gets ||b - A x|| / ||b||
 * over the same rows. */
int afo_pcg_jacobi(int n, const int32_t* row_ptr, const int32_t* cols, const double* values, const double* b,
                   double* x, double rtol, int max_iter, const uint8_t* norm_skip, double* relres, int nb_threads);

/* Wall-clock seconds (monotonic). */
double afo_wtime(void);
int afo_max_threads(void);

/* CPU baselines (afem_oracle_dok.cc, afem_oracle.c): the reference's DOK
 * assembly (ordered map, zeros skipped) of cells [0, nb_cell), Poisson P1;
 * returns the stored entries or -1 when cap is too small.  And the node-wise
 * sparsity on nb_threads threads (ascending columns): per node, the nodes of
 * its incident cells, sorted and deduplicated; returns nnz or -1 (cap). */
int64_t afo_assemble_dok(int kind, int nb_node, int nb_cell, const double* coords, const int32_t* cell_nodes,
                         int32_t* row_ptr, int32_t* cols, double* values, int64_t cap);
int64_t afo_sparsity_nodewise(int nb_node, int npc, const int32_t* cell_nodes, const int32_t* nc_ptr,
                              const int32_t* nc_cell, int32_t* row_ptr, int32_t* cols, int64_t cap, int nb_threads);

#ifdef __cplusplus
}
#endif
#endif
