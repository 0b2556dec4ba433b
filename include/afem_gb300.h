/*
 * afem_gb300.h -- C ABI of the GB300 (sm_103a) node-wise P1 assembly and
 * Krylov library.
 *
 * This is the drop-in boundary for ArcaneFEM's GPU hot path.  Each entry
 * point names the reference interface it replaces (paths relative to the
 * arcanefem source tree).  Conventions:
 *
 *   - every pointer argument suffixed _d is device memory; _h is host memory;
 *   - every call is asynchronous on the stream of its context, except where
 *     it returns a host value (documented per call);
 *   - every call returns an afem_status and never aborts; the message of the
 *     last failure of the calling thread is afem_last_error();
 *   - coords: double[nb_node][3] (Arcane Real3, z = 0 in 2D);
 *     cell_nodes: int32[nb_cell][nodes_per_cell] (3 triangle, 4 tetrahedron);
 *   - DoF numbering: dof = node * nb_dof + component
 *     (femutils/FemDoFsOnNodes.cc:72-112);
 *   - row_ptr: int32[nb_row + 1].  The reference CsrFormatMatrixView stores N
 *     row starts and ends the last row at nbColumn()
 *     (femutils/CsrFormatMatrixView.h:181-187); row_ptr[N] = nnz is that end.
 *
 * Handles are not thread safe: use one context per host thread / stream.
 */
#ifndef AFEM_GB300_H
#define AFEM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The library is built with hidden visibility; these are its only exports. */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ---------------------------------------------------------------------- */
/* Status codes.  Replace ARCANE_FATAL / ARCANE_THROW (femutils/BSRFormat.cc:51-55)
 * and the HYPRE error mapping (femutils/HypreDoFLinearSystem.cc:86-111). */
typedef int afem_status;
enum {
  AFEM_OK = 0,
  AFEM_ERR_BAD_ARG = 1,          /* ArgumentException */
  AFEM_ERR_OOM = 2,
  AFEM_ERR_NOT_CONVERGED = 3,
  AFEM_ERR_BREAKDOWN = 4,        /* <p, A p> <= 0 or NaN in CG */
  AFEM_ERR_TIMEOUT = 5,          /* a bounded device wait ran out */
  AFEM_ERR_CUDA = 6,
  AFEM_ERR_MESH = 7,             /* bad connectivity, degree above a kernel limit */
  AFEM_ERR_NOT_IMPLEMENTED = 8,  /* NotImplementedException */
  AFEM_ERR_NOT_FOUND = 9         /* "Value not found" (BSRFormat.cc:105) */
};

/* Message of the last failure on this host thread ("" if none). */
const char* afem_last_error(void);
/* Library version, e.g. 10000 for 1.0.0. */
int afem_version(void);

/* ---------------------------------------------------------------------- */
/* Context: a stream plus a device scratch arena.  Replaces the Arcane
 * RunQueue and its memory resource (femutils/CsrFormatMatrix.cc:40-47). */
typedef struct afem_context_s* afem_context;

afem_status afem_context_create(afem_context* ctx, void* cuda_stream);
afem_status afem_context_destroy(afem_context ctx);
afem_status afem_context_set_stream(afem_context ctx, void* cuda_stream);
/* Block the host until the context's stream is idle (RunQueue::barrier). */
afem_status afem_context_synchronize(afem_context ctx);
/* Number of kernels this library launched through the context so far. */
afem_status afem_context_launch_count(afem_context ctx, int64_t* count_h);
/* Measured FP64 FMA issue rate of the device (G FMA/s), the ceiling of the
 * FP64-bound element kernels.  No reference counterpart (a roofline helper).
 * Synchronous, about 10 ms. */
afem_status afem_device_fp64_fma_rate(afem_context ctx, double* gfma_per_s_h);

/* ---------------------------------------------------------------------- */
/* Connectivity and sparsity.
 *
 * Node -> cell adjacency: Arcane's nodeCell() connectivity
 * (used at femutils/BSRFormat.h:411,428; NodeWiseCsrBiliAssembly.cc:179,188),
 * cells ascending per node.  nc_local_d[p] = position of the node inside
 * cell nc_cell_d[p]; nc_inverse_d[cell*nodes_per_cell + i] = p, the incidence
 * of (cell, local node i) in that list (nullable).  Buffers:
 * nc_ptr_d[nb_node+1], nc_cell_d, nc_local_d and
 * nc_inverse_d[nb_cell*nodes_per_cell].  Deterministic.  nodes_per_cell:
 * 3 or 4 for cells; 2 also serves boundary edges (node -> face lists). */
afem_status afem_node_cell_build(afem_context ctx, int nb_node, int nb_cell, int nodes_per_cell,
                                 const int32_t* cell_nodes_d, int32_t* nc_ptr_d, int32_t* nc_cell_d,
                                 uint8_t* nc_local_d, int32_t* nc_inverse_d);

/* Column order of a row. */
enum {
  AFEM_COLS_ASCENDING = 0,   /* canonical; the DOK/ordered-map order (internal/OrderedRowColumnMap.h:59) */
  AFEM_COLS_SELF_LAST = 1    /* neighbours ascending, diagonal last (BSRFormat.cc:658-672,758-770) */
};

/* Node-to-node sparsity, step 1: row_ptr_d[nb_node+1] (row length = 1 +
 * number of distinct neighbours) and the total in *nnz_h (host, synchronous).
 * A row of more than 255 entries (the slot map below is uint8) or a node id
 * outside [0, nb_node) returns AFEM_ERR_MESH. nodes_per_cell: 3, 4 or 8.
 * The pass that counts the rows also finds their columns and the slot map;
 * the context keeps them for the next afem_sparsity_cols on the same
 * cell_nodes_d / nc_ptr_d / nc_cell_d, which then only copies them into
 * place.  Their buffer (about 4 (nodes_per_cell - 1) + nodes_per_cell bytes
 * per incidence: 0.8 GB for 12.6 M tetrahedra) grows as needed and stays
 * with the context until afem_context_destroy; without room for it the
 * rows are counted alone and afem_sparsity_cols finds them again.  The mesh
 * arrays must not change between the two calls (as row_ptr_d already
 * requires).
 * Replaces computeRowIndexAtomicFree / computeRowIndex (BSRFormat.cc:562-573,
 * 912-924) and _buildOffsetsNodeWiseCsr (NodeWiseCsrBiliAssembly.cc:90-112). */
afem_status afem_sparsity_rows(afem_context ctx, int nb_node, int nodes_per_cell, const int32_t* cell_nodes_d,
                               const int32_t* nc_ptr_d, const int32_t* nc_cell_d, int32_t* row_ptr_d,
                               int64_t* nnz_h);
/* Step 2: cols_d[nnz] in the requested order, and nc_slot_d[nb_cell *
 * nodes_per_cell * nodes_per_cell] (uint8): for incidence p of node n and
 * cell node j, the position inside row n of column cell_nodes[c][j].  The
 * slot map lets the assembly skip the reference's linear column search
 * (BSRFormat.h:449-462).  After afem_sparsity_rows on other mesh arrays (or
 * without the kept rows) the columns are found again here.  Replaces
 * computeColumnsAtomicFree / computeColumns (BSRFormat.cc:578-772, 929-971)
 * and _buildMatrixNodeWiseCsr (NodeWiseCsrBiliAssembly.cc:115-152). */
afem_status afem_sparsity_cols(afem_context ctx, int nb_node, int nodes_per_cell, const int32_t* cell_nodes_d,
                               const int32_t* nc_ptr_d, const int32_t* nc_cell_d, const uint8_t* nc_local_d,
                               const int32_t* row_ptr_d, int col_order, int32_t* cols_d, uint8_t* nc_slot_d);

/* ---------------------------------------------------------------------- */
/* Node-wise (atomic-free) assembly.
 *
 * Value layouts for block size b (BSRFormat.h:514-526, BSRFormat.cc:79-106):
 *   AFEM_LAYOUT_PER_BLOCK: values[(row_ptr[r] + x) * b*b + i*b + j]
 *   AFEM_LAYOUT_PER_ROW  : values[row_ptr[r]*b*b + b*(x + i*nnzb_row) + j]
 *                          (CSR-compatible: scalar row r*b+i is contiguous)
 * For b = 1 both layouts are plain CSR. */
enum { AFEM_LAYOUT_PER_BLOCK = 0, AFEM_LAYOUT_PER_ROW = 1 };

typedef struct {
  int dim;                       /* 2 (triangles) or 3 (tetrahedra) */
  int nb_node;
  int nb_cell;
  const double* coords_d;        /* [nb_node][3] */
  const int32_t* cell_nodes_d;   /* [nb_cell][dim+1] */
  const int32_t* nc_ptr_d;       /* [nb_node+1] */
  const int32_t* nc_cell_d;      /* [nb_cell*(dim+1)] */
  const uint8_t* nc_local_d;     /* [nb_cell*(dim+1)] */
  const uint8_t* nc_slot_d;      /* [nb_cell*(dim+1)^2] from afem_sparsity_cols */
  const int32_t* nc_inverse_d;   /* [nb_cell*(dim+1)] from afem_node_cell_build */
} afem_mesh_view;

/* Element arithmetic of the assembly kernels (per context; default
 * AFEM_FORMULATION_REFERENCE).
 *   REFERENCE: the reference's element functions in their own operation order,
 *     every product and sum rounded separately as its CPU build evaluates them
 *     (modules/poisson/ElementMatrix.h:54-63,107-118,
 *     modules/poisson/ElementMatrixHexQuad.h:63-91,239-266,
 *     modules/elasticity/ElementMatrix.h:216-301, with the geometry of
 *     femutils/ArcaneFemFunctionsGpu.h:76-128,241-281,414-610).  Assembled
 *     values are bit-identical to the reference's node-wise assembly.
 *   TESTLAB: the testlab B-matrix form of the P1 Poisson element
 *     (modules/testlab/FemModule.h:469-538, NodeWiseCsrBiliAssembly.cc:
 *     194-211,269-290), bit-identical to testlab's nwcsr path; the other
 *     element kinds use REFERENCE.
 *   MINIMAL: the same matrices with the fewest FP64 instructions (edge-vector
 *     cofactors, zero row sums, per-cell Jacobian moments): 2-3x faster on
 *     GB300's narrow FP64 pipe and about 25x closer to exact arithmetic than
 *     the reference's own formula, so NOT bit-identical to it (within
 *     1e-11 of an entry near 1e-3 of its row maximum on 128^3 meshes).
 * No reference counterpart (the reference has one formulation per path). */
enum { AFEM_FORMULATION_REFERENCE = 0, AFEM_FORMULATION_TESTLAB = 1, AFEM_FORMULATION_MINIMAL = 2 };
afem_status afem_context_set_element_formulation(afem_context ctx, int formulation);
afem_status afem_context_get_element_formulation(afem_context ctx, int* formulation_h);

/* Degenerate cells.  Every element kernel checks its cell's measure (tet 6V,
 * triangle 2A, Jacobian determinant at each Gauss point); a zero, subnormal or
 * non-finite one sets a flag in the context, and the next synchronous call
 * (afem_context_synchronize, afem_assemble_to_host, afem_assemble_host_io,
 * afem_gather_to_host) returns AFEM_ERR_MESH and clears it.  The reference
 * divides by the measure without a check (ArcaneFemFunctionsGpu.h:113-128,
 * 414-535) and yields non-finite entries; the values here are the same, but
 * the status says so. */

/* Scalar Poisson P1 stiffness, -div(k grad u): values_d[nnz] (CSR) receives
 * sum_cells k_c vol grad N_i . grad N_j.  cell_coeff_d (nullable) holds k_c.
 * Replaces assembleBilinearAtomicFree with _computeElementVectorTria3Gpu /
 * _computeElementVectorTetra4Gpu (BSRFormat.h:556-565,
 * modules/poisson/ElementMatrix.h:54-63,107-118) and the testlab
 * _assembleNodeWiseCsrBilinearOperatorTria3/Tetra4
 * (modules/testlab/NodeWiseCsrBiliAssembly.cc:157-297).  Overwrites
 * values_d (no prior zeroing needed).  Uses scratch from the context. */
afem_status afem_assemble_poisson_p1(afem_context ctx, const afem_mesh_view* mesh, const int32_t* row_ptr_d,
                                     const double* cell_coeff_d, double* values_d);

/* Bilinear / trilinear Lagrange Poisson stiffness (Quad4 for dim 2, Hexa8 for
 * dim 3: the view's cell arrays hold 2^dim nodes per cell in the reference
 * element's order -- quads counter-clockwise, hexahedra the bottom face
 * counter-clockwise then the top face), 2 x 2 (x 2) Gauss points:
 * _computeElementVectorQuad4Gpu / _computeElementVectorHexa8Gpu
 * (modules/poisson/ElementMatrixHexQuad.h:63-91,239-266).  The node -> cell
 * incidence, slot map and CSR structure come from afem_node_cell_build /
 * afem_sparsity_* with nodes_per_cell = 2^dim.  Element matrices are computed
 * once per cell into ke[npc * npc * nb_cell] (afem_element_matrices_poisson_q1),
 * then gathered node-wise (afem_gather_poisson_q1); afem_assemble_poisson_q1
 * does both with library scratch. */
afem_status afem_element_matrices_poisson_q1(afem_context ctx, const afem_mesh_view* mesh, const double* cell_coeff_d,
                                             double* ke_d);
afem_status afem_gather_poisson_q1(afem_context ctx, const afem_mesh_view* mesh, const int32_t* row_ptr_d,
                                   const double* ke_d, double* values_d);
afem_status afem_assemble_poisson_q1(afem_context ctx, const afem_mesh_view* mesh, const int32_t* row_ptr_d,
                                     const double* cell_coeff_d, double* values_d);

/* Linear elasticity P1 tetrahedra, 3x3 blocks (b = 3):
 * values_d[nnzb * 9] in the given layout.  Replaces assembleBilinearAtomicFree
 * with computeElementVectorTetra4Gpu (modules/elasticity/ElementMatrix.h:216-301,
 * modules/elasticity/FemModule.cc:257-271).  Uses scratch from the context. */
afem_status afem_assemble_elasticity_tet4(afem_context ctx, const afem_mesh_view* mesh, const int32_t* row_ptr_d,
                                          double lambda, double mu, int layout, double* values_d);

/* The two stages of the assemblies above, for callers that keep the element
 * matrices themselves (and to time the stages separately).  Stage 1 computes
 * each element matrix once per cell and stores its rows in incidence order:
 * row i of cell c goes to incidence p = nc_inverse[c*npc + i], at
 * ke_d[p*npc .. p*npc + npc-1] (Poisson, npc = dim+1 values) or
 * ke_d[p*36 + a*12 + 3*m + b] (elasticity: the 3x12 row block, rows a,
 * column node m, component b).  Size: nb_cell*npc*npc doubles (Poisson),
 * nb_cell*144 (elasticity).  Stage 2 streams, per row, the contiguous
 * element rows of the incident cells in increasing cell order (no atomics). */
afem_status afem_element_matrices_poisson_p1(afem_context ctx, const afem_mesh_view* mesh,
                                             const double* cell_coeff_d, double* ke_d);
afem_status afem_gather_poisson_p1(afem_context ctx, const afem_mesh_view* mesh, const int32_t* row_ptr_d,
                                   const double* ke_d, double* values_d);
afem_status afem_element_matrices_elasticity_tet4(afem_context ctx, const afem_mesh_view* mesh, double lambda,
                                                  double mu, double* ke_d);
afem_status afem_gather_elasticity_tet4(afem_context ctx, const afem_mesh_view* mesh, const int32_t* row_ptr_d,
                                        const double* ke_d, int layout, double* values_d);

/* Gather and copy back in one call: the node-wise gather runs in `chunks`
 * (1..16; 0 = one range per ~80 MB of values, at most 12) node ranges on
 * the context stream, and each finished range of
 * values_d goes to the host buffer values_h on a second stream while the next
 * range is gathered (pinned values_h for a real overlap).  kind selects the
 * gather of afem_gather_poisson_p1, afem_gather_poisson_q1 or
 * afem_gather_elasticity_tet4 (layout used by the latter only).  Returns when
 * values_h holds the whole matrix.  For callers that need the values on the
 * host, as the reference's CPU-side linear systems do
 * (femutils/CsrDoFLinearSystemImpl.cc, HypreDoFLinearSystem.cc:596-751). */
#define AFEM_GATHER_POISSON_P1 0
#define AFEM_GATHER_POISSON_Q1 1
#define AFEM_GATHER_ELASTICITY_TET4 2
afem_status afem_gather_to_host(afem_context ctx, const afem_mesh_view* mesh, int kind, const int32_t* row_ptr_d,
                                const double* ke_d, int layout, double* values_d, double* values_h, int chunks);
/* The whole values assembly with the copy back pipelined: the cells are
 * split into `chunks` (1..16; 0 = one range per ~80 MB of values, at most
 * 12) ranges; after the element matrices of each
 * range, the nodes it completes (a prefix of the node numbering: every
 * incident cell done) are gathered and their values copied to values_h on a
 * second stream while the next range computes.  kind: AFEM_GATHER_POISSON_P1
 * or AFEM_GATHER_POISSON_Q1 (cell_coeff_d nullable) or
 * AFEM_GATHER_ELASTICITY_TET4 (lambda, mu, layout).  ke_d is the caller's element buffer (afem_element_matrices_*
 * sizes).  Returns when values_h holds the whole matrix; values_d holds it
 * too.  Meshes numbered so that nodes complete late overlap less. */
afem_status afem_assemble_to_host(afem_context ctx, const afem_mesh_view* mesh, int kind, const int32_t* row_ptr_d,
                                  const double* cell_coeff_d, double lambda, double mu, int layout, double* ke_d,
                                  double* values_d, double* values_h, int chunks);
/* afem_assemble_to_host with the node coordinates coming from the host too:
 * coords_h [nb_node][3] (pinned for overlap) is copied into mesh->coords_d
 * in node prefixes on a third stream, each prefix ahead of the first cell
 * range whose cells use it (a node is needed from the range of its first
 * incident cell on), while earlier ranges compute.  Host coordinates in, host
 * values out; meshes numbered so that cells use nodes in order overlap most. */
afem_status afem_assemble_host_io(afem_context ctx, const afem_mesh_view* mesh, const double* coords_h, int kind,
                                  const int32_t* row_ptr_d, const double* cell_coeff_d, double lambda, double mu,
                                  int layout, double* ke_d, double* values_d, double* values_h, int chunks);

/* Allocation-free assembly of the scalar Poisson P1 matrix.  No counterpart
 * in the reference: it serves callers that cannot let a library allocate
 * device memory (a host framework that owns all device allocations through
 * its own pool and budgets them, or a step loop that cannot afford the
 * synchronisation a device allocation implies).  Same arguments and results
 * as afem_assemble_poisson_p1, but no
 * context: the work runs on cuda_stream, and the element-row scratch is a
 * fixed 32 MiB device array inside the library, held by every GPU that loads
 * the library until the process exits.  Limit: 4,194,304 doubles of scratch,
 * i.e. at most 262,144 tetrahedra or 466,033 triangles; larger meshes are
 * rejected with AFEM_ERR_BAD_ARG.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress) for that device: make that
 * first call before any stream capture.  All calls share the one array, so
 * calls that can overlap on the GPU (different streams, or different host
 * threads without ordering) race and must be serialised by the caller.  The
 * stream's device must be the current device (AFEM_ERR_BAD_ARG otherwise).
 * Element arithmetic: AFEM_FORMULATION_REFERENCE; no context, hence no
 * degenerate-cell status. */
afem_status afem_assemble_poisson_p1_noalloc(void* cuda_stream, const afem_mesh_view* mesh,
                                             const int32_t* row_ptr_d, const double* cell_coeff_d,
                                             double* values_d);

/* Expand block-row pointers / block columns of a b x b BSR to scalar CSR
 * row_ptr_d[nb_node*b+1] and cols_d[nnzb*b*b] (the per-row value layout is
 * already CSR-ordered).  Replaces the host loops of BSRMatrix::toCsr
 * (femutils/BSRFormat.cc:110-172). */
afem_status afem_bsr_to_csr_structure(afem_context ctx, int nb_block_row, int b, const int32_t* brow_ptr_d,
                                      const int32_t* bcols_d, int32_t* row_ptr_d, int32_t* cols_d);

/* rhs_d[node*nb_dof] = sum_cells qdot * measure / (dim+1), other entries
 * untouched.  Replaces applyConstantSourceToRhsBase
 * (femutils/ArcaneFemFunctionsGpu.h:676-708). */
afem_status afem_rhs_constant_source(afem_context ctx, const afem_mesh_view* mesh, double qdot, int nb_dof,
                                     double* rhs_d);

/* Body force on tetrahedra, rhs_d[3*node + k] += sum_cells f[k] * vol / 4,
 * node-wise (no atomics).  Replaces the host loop of
 * FemModuleElasticity::_applyBodyForce (modules/elasticity/BodyForce.h:148-160). */
/* Constant source on Quad4 / Hexa8 cells (2^dim nodes, as
 * afem_assemble_poisson_q1): rhs[n nb_dof] = sum over the incident cells of
 * sum_gp N_n qdot w detJ, 2 x 2 (x 2) Gauss points
 * (applyConstantSourceToRhsQuad4 / Hexa8, femutils/ArcaneFemFunctionsGpu.cc:
 * 393-458,875-960, which adds with atomics; here per (cell, node) then per
 * node in increasing cell order). */
afem_status afem_rhs_constant_source_q1(afem_context ctx, const afem_mesh_view* mesh, double qdot, int nb_dof,
                                        double* rhs_d);
afem_status afem_rhs_body_force_tet4(afem_context ctx, const afem_mesh_view* mesh, double fx, double fy, double fz,
                                     double* rhs_d);

/* Boundary-face right-hand-side terms on P1 meshes (boundary edges in 2D,
 * triangles in 3D), added into rhs:
 *   AFEM_FACE_SCALAR  scalar Neumann flux:  rhs[dof(n, 0)] += g[0] |f| / nf
 *   AFEM_FACE_NORMAL  vector Neumann flux:  rhs[dof(n, 0)] += (nrm . g) |f| / nf
 *   AFEM_FACE_VECTOR  traction:             rhs[dof(n, c)] += g[c] |f| / nf, c < dim
 * |f| = edge length or triangle area, nf = dim nodes per face, dof(n, c) =
 * n nb_dof + c, nrm = unit outward normal: the face's node order as given
 * when outward_d[f] != 0 (Arcane's isSubDomainBoundaryOutside), its first two
 * nodes swapped otherwise (outward_d null: all outward).  g_h: host array of
 * dim values ("NULL" components = 0).  Replaces applyNeumannToRhsTria3 /
 * Tetra4 (femutils/ArcaneFemFunctionsGpu.cc:679-735,1082-1140, atomic adds)
 * and applyTractionToRhsTria3 / Tetra4 (femutils/ArcaneFemFunctions.h:
 * 2854-2885,2188-2220): contributions are gathered node-wise in increasing
 * face order, so the result is deterministic and equals the sequential
 * face-loop order. */
#define AFEM_FACE_SCALAR 0
#define AFEM_FACE_NORMAL 1
#define AFEM_FACE_VECTOR 2
afem_status afem_rhs_boundary_faces(afem_context ctx, int dim, int nb_node, int nb_face, const double* coords_d,
                                    const int32_t* face_nodes_d, const uint8_t* outward_d, int mode,
                                    const double* g_h, int nb_dof, double* rhs_d);

/* ---------------------------------------------------------------------- */
/* Linear system: mirrors CsrDoFLinearSystemImpl
 * (femutils/internal/CsrDoFLinearSystemImpl.h:36-113) behind
 * IDoFLinearSystemImpl (femutils/internal/IDoFLinearSystemImpl.h:37-70).
 * It owns the DoF variables (rhs, solution, forced info/value, elimination
 * info/value) and keeps a NON-owning view of the CSR matrix set by
 * afem_ls_set_csr_values, which must stay valid until afem_ls_solve
 * (femutils/DoFLinearSystem.h:318-328). */
typedef struct afem_linear_system_s* afem_linear_system;

enum { AFEM_ELIMINATE_NONE = 0, AFEM_ELIMINATE_ROW = 1, AFEM_ELIMINATE_ROW_COLUMN = 2 }; /* FemUtilsGlobal.h:51-62 */

/* IDoFLinearSystemFactory::createInstance (femutils/IDoFLinearSystemFactory.h:42-43). */
afem_status afem_ls_create(afem_context ctx, int nb_dof, afem_linear_system* ls);
afem_status afem_ls_destroy(afem_linear_system ls);
/* setCSRValues (CsrDoFLinearSystemImpl.h:98-101). */
afem_status afem_ls_set_csr_values(afem_linear_system ls, const int32_t* row_ptr_d, const int32_t* cols_d,
                                   double* values_d, int64_t nnz);
/* setCSRValues(const CSRFormatView&) with the reference's view as it is
 * (femutils/CsrFormatMatrixView.h:135-210, filled by
 * femutils/CsrFormatMatrix.cc:35-95): rows_d[nb_row] holds each row's first
 * slot, with NO trailing entry (the last row ends at nb_column, the view's
 * nbColumn(), :181-187); rows_nb_column_d[nb_row] (nullable) holds each row's
 * slot count (nbColumnForRow); columns_d[nb_column] may hold -1 in unused
 * slots (CsrFormatMatrix.cc:49-50), which every kernel of the library skips:
 * the transformations as the reference's (column_index > 0 / >= 0 tests,
 * CsrDoFLinearSystemImpl.cc:111,217), the SpMVs and solves as absent
 * entries.  Rows must start at non-decreasing offsets; slots past a row's
 * count up to the next row's start must be -1.  No copy of the matrix is
 * made: the library keeps a device array of the nb_row + 1 row offsets
 * (checked when set; synchronous) and a non-owning view of columns and
 * values, valid until afem_ls_solve.  nb_row must equal the system's DoF
 * count (the compacted DoF family of CsrDoFLinearSystemImpl.cc:27-29).
 * rows_nb_column_d = NULL takes each row's count as its range size, which is
 * what CsrFormat::translateToLinearSystem stores.  The learned
 * preconditioner and block_size = 3 need a view without unused slots
 * (AFEM_ERR_NOT_IMPLEMENTED / AFEM_ERR_BAD_ARG otherwise). */
afem_status afem_ls_set_csr_view(afem_linear_system ls, int32_t nb_row, const int32_t* rows_d,
                                 const int32_t* rows_nb_column_d, int64_t nb_column, const int32_t* columns_d,
                                 double* values_d);
/* hasSetCSRValues / getCSRValues. */
afem_status afem_ls_get_csr_values(afem_linear_system ls, const int32_t** row_ptr_d, const int32_t** cols_d,
                                   double** values_d, int64_t* nnz);
/* Device pointers to the DoF variables: rhsVariable, solutionVariable,
 * getForcedInfo (uint8 0/1), getForcedValue, getEliminationInfo,
 * getEliminationValue (DoFLinearSystemImplBase.cc:27-36). */
afem_status afem_ls_dof_variables(afem_linear_system ls, double** rhs_d, double** solution_d, uint8_t** forced_info_d,
                                  double** forced_value_d, uint8_t** elimination_info_d,
                                  double** elimination_value_d);
/* clearValues (DoFLinearSystemImplBase.cc:44-50, CsrDoFLinearSystemImpl.h:90-95). */
afem_status afem_ls_clear_values(afem_linear_system ls);
/* matrixAddValue / matrixSetValue (CsrDoFLinearSystemImpl.h:55-65): one entry,
 * linear search in the row; AFEM_ERR_NOT_FOUND if the column is not stored. */
afem_status afem_ls_matrix_add_value(afem_linear_system ls, int32_t row, int32_t col, double value);
afem_status afem_ls_matrix_set_value(afem_linear_system ls, int32_t row, int32_t col, double value);
/* eliminateRow / eliminateRowColumn throw NotImplementedException on the CSR
 * impl (CsrDoFLinearSystemImpl.h:67-75): AFEM_ERR_NOT_IMPLEMENTED here too. */
afem_status afem_ls_eliminate_row(afem_linear_system ls, int32_t row, double value);
afem_status afem_ls_eliminate_row_column(afem_linear_system ls, int32_t row, double value);

/* Dirichlet flagging on a node group (nodes_d[nb_sel]):
 * applyDirichletToNodeGroupViaPenalty (ArcaneFemFunctionsGpu.cc:54-78):
 *   forced_info = 1, forced_value = penalty, rhs = penalty * value;
 * applyDirichletToNodeGroupViaRowOrRowColumnElimination (ArcaneFemFunctionsGpu.cc:83-105):
 *   elimination_info = type, elimination_value = value. */
afem_status afem_dirichlet_penalty(afem_linear_system ls, int nb_sel, const int32_t* nodes_d, int nb_dof_per_node,
                                   int dof_index, double value, double penalty);
afem_status afem_dirichlet_elimination(afem_linear_system ls, int elimination_type, int nb_sel,
                                       const int32_t* nodes_d, int nb_dof_per_node, int dof_index, double value);

/* applyMatrixTransformation (CsrDoFLinearSystemImpl.cc:235-242): keeps the
 * pre-elimination values needed for row-column elimination, applies row
 * elimination, row-column elimination (with the reference's column_index > 0
 * test, :111) and forced (penalty) diagonals.  Fully on the device. */
afem_status afem_ls_apply_matrix_transformation(afem_linear_system ls);
/* applyRHSTransformation (CsrDoFLinearSystemImpl.cc:247-253 and
 * DoFLinearSystemImplBase.cc:55-88): rhs_j -= A_ij g_i for row-column
 * eliminated i in increasing i (the host std::map order of the reference),
 * then rhs_i = g_i on eliminated rows.  Fully on the device. */
afem_status afem_ls_apply_rhs_transformation(afem_linear_system ls);

/* ---------------------------------------------------------------------- */
/* Krylov solve. */
enum { AFEM_PRECOND_NONE = 0, AFEM_PRECOND_JACOBI = 1, AFEM_PRECOND_LEARNED = 2 };
enum { AFEM_PRECISION_FP64 = 0, AFEM_PRECISION_MIXED = 1 };

typedef struct {
  double rtol;            /* stop when ||b - A x|| <= max(rtol ||b||, atol) (two-norm, HypreDoFLinearSystem.cc:596-603) */
  double atol;
  int max_iter;           /* default 1000 when 0 (HypreDoFLinearSystem.cc:182) */
  int precond;            /* AFEM_PRECOND_* */
  int precision;          /* AFEM_PRECISION_*; MIXED = FP32 inner CG inside FP64 iterative refinement */
  int skip_forced_rows;   /* leave penalty (forced) rows out of both norms of the stop test */
  double inner_rtol;      /* MIXED and batch: FP32 residual reduction between reliable updates
                             (<= 0: 0.1) */
  int check_every;        /* iterations between host convergence checks (default 16) */
  int block_size;         /* MIXED: 3 = the CSR holds 3x3 blocks (the per-row layout of a 3-DoF
                             BSR matrix): the FP32 SpMV then reads one column index per block
                             (the FP32 BSR SpMV); 0 or 1: scalar rows */
} afem_solver_options;

typedef struct {
  int iterations;         /* total (inner) CG iterations */
  int refinements;        /* outer FP64 refinement steps (MIXED) */
  int status;             /* afem_status of the solve */
  double relres;          /* true FP64 ||b - A x|| / ||b|| recomputed at the end */
  double solve_ms;        /* device time of the solve */
} afem_solve_info;

void afem_solver_options_default(afem_solver_options* opt);

/* x_d (initial guess in, solution out) for the CSR system (row_ptr, cols, values).
 * Replaces IDoFLinearSystemImpl::solve of the HYPRE / PETSc / Aleph / Arcane
 * MatVec backends (HypreDoFLinearSystem.cc:265-858, DoFLinearSystem.cc:146-159).
 * forced_info_d (nullable) marks rows left out of the stop test when
 * opt->skip_forced_rows.  Synchronous (returns after convergence). */
afem_status afem_cg_solve_csr(afem_context ctx, int n, const int32_t* row_ptr_d, const int32_t* cols_d,
                              const double* values_d, const double* b_d, double* x_d, const uint8_t* forced_info_d,
                              const afem_solver_options* opt, afem_solve_info* info);

/* IDoFLinearSystemImpl::solve: solves the linear system's matrix view for
 * its rhs into its solution variable (applyLinearSystemTransformationAndSolve
 * calls the two transformations first, femutils/DoFLinearSystem.cc:487-493).
 * opt->precond = AFEM_PRECOND_LEARNED runs the flexible CG with the network
 * attached by afem_ls_set_learned_preconditioner (its operator is refreshed
 * from the system's matrix whenever the values changed since its last use);
 * the other preconditioners run the CG of afem_cg_solve_csr.  Failure
 * statuses (AFEM_ERR_NOT_CONVERGED with the last iterate in the solution,
 * AFEM_ERR_BREAKDOWN) fill *info too. */
afem_status afem_ls_solve(afem_linear_system ls, const afem_solver_options* opt, afem_solve_info* info);

/* y = A x, FP64 CSR. */
afem_status afem_spmv_csr(afem_context ctx, int n, const int32_t* row_ptr_d, const int32_t* cols_d,
                          const double* values_d, const double* x_d, double* y_d);

/* ---------------------------------------------------------------------- */
/* Learned preconditioner.  No counterpart in the reference (it delegates to
 * HYPRE BoomerAMG / PETSc / Aleph): one symmetric V(1,1)-cycle of geometric
 * multigrid on the Galerkin hierarchy A_{l+1} = P_l^T A_l P_l, with
 * weighted-Jacobi smoothers whose per-node weights
 *   d_l = cap_l * sigmoid(c_l + logit 0.8),  cap_l = 2 / sum_j |A_l,ij|
 * come from a message-passing network on the mesh graph (6 layers, width 64,
 * BF16 GEMMs on the tcgen05 tensor cores with FP32 accumulation in TMEM and
 * TMA-loaded operand tiles), trained on the GPU with this library's forward
 * and backward kernels and applied inside flexible CG.  The GEMMs' mbarrier
 * waits are bounded: a wait that runs out is reported as AFEM_ERR_TIMEOUT by
 * the call that ran the network.
 * The cap keeps the V-cycle symmetric positive definite for any network
 * output; with c = 0 the smoother is l1-Jacobi at 0.8 of the cap.
 * On the finest level and on every level of at most 2048 rows the smoother
 * is a learned factored sparse approximate inverse instead of d_l * x:
 *   G_l = theta_l L_l^T L_l,  L_l = (I + N_l) diag(sqrt d_l),
 *   N_l,ij = m_ij sqrt(d_i d_j) A_l,ij  (strictly lower pattern of A_l),
 *   m_ij = 2 tanh(ew_l . (o_i * o_j) + eb_l)  (an edge head on the level's
 *   network output), theta_l = 1.9 / max(1.9, max_i sum_j |(L^T L A_l)_ij|):
 * SPD by construction and with lambda_max(G_l A_l) < 2, so the V-cycle stays
 * SPD; theta_l takes part in the gradient through the row that attains the
 * bound.  Zero edge heads give the weighted-Jacobi smoother exactly.
 * The first level below the finest of at most 320 rows is solved exactly:
 * the V-cycle stops there and applies the inverse of the block of that
 * level's nonzero rows (FP64 Cholesky on the host in afem_mpnn_set_operator,
 * applied in FP32); the levels below it are not used, and afem_mpnn_set_operator
 * returns AFEM_ERR_BREAKDOWN if that block is not positive definite.  The
 * factored levels are the finest and those of at most 2048 rows above it.
 *
 * The caller provides the level hierarchy as device CSR matrices (FP32
 * weights): graph[l] (level l adjacency, symmetric; level 0 = the matrix
 * graph, its weights are set from A by afem_mpnn_set_operator and graph_w[0]
 * is ignored), restr[l] (level l -> l+1, feature restriction), prol[l]
 * (level l+1 -> l, the multigrid prolongation), their transposes, and the
 * sparsity pattern of every coarse operator (coarse_rp[l], coarse_cols[l]
 * for l >= 1; entry 0 is ignored) that must hold all entries of
 * P_{l-1}^T A_{l-1} P_{l-1}.  The pointer arrays are host arrays of device
 * pointers. */
typedef struct afem_mpnn_s* afem_mpnn;

afem_status afem_mpnn_create(afem_context ctx, int nb_levels, int nb_layers, const int* level_rows_h,
                             const int32_t* const* graph_rp_h, const int32_t* const* graph_cols_h,
                             const float* const* graph_w_h, const int32_t* const* restr_rp_h,
                             const int32_t* const* restr_cols_h, const float* const* restr_w_h,
                             const int32_t* const* restrT_rp_h, const int32_t* const* restrT_cols_h,
                             const float* const* restrT_w_h, const int32_t* const* prol_rp_h,
                             const int32_t* const* prol_cols_h, const float* const* prol_w_h,
                             const int32_t* const* prolT_rp_h, const int32_t* const* prolT_cols_h,
                             const float* const* prolT_w_h, const int32_t* const* coarse_rp_h,
                             const int32_t* const* coarse_cols_h, int max_batch, afem_mpnn* net);
afem_status afem_mpnn_destroy(afem_mpnn net);
/* nb_layers (1..nb_levels) message-passing layers run on levels
 * 0..nb_layers-1; deeper levels take the restricted output of the last layer.
 * Number of FP32 parameters.  Flat layout: W_in[2][64], b_in[64]; per layer
 * W1[64][64], W2[64][64], b[64]; then per level a head w[64], beta; then per
 * factored level (level 0 and the levels of at most 2048 rows above the
 * exact level, in level order) an edge head ew[64], eb.  Heads of levels at
 * or below the exact level stay in the layout with zero gradients. */
int afem_mpnn_param_count(afem_mpnn net);
afem_status afem_mpnn_set_params(afem_mpnn net, const float* params_d);
afem_status afem_mpnn_get_params(afem_mpnn net, float* params_d);
/* Diagonal, level-0 edge weights -A_ij / sqrt(A_ii A_jj), coefficient
 * features, the Galerkin coarse operators and the smoother caps from the
 * FP64 CSR operator (same graph as level 0).  Synchronous (one host
 * reduction of log diag A); AFEM_ERR_BAD_ARG when a coarse pattern misses
 * entries. */
afem_status afem_mpnn_set_operator(afem_mpnn net, int n, const int32_t* row_ptr_d, const int32_t* cols_d,
                                   const double* values_d);
/* z = M r for `batch` FP32 vectors stored one after the other. */
afem_status afem_mpnn_forward(afem_mpnn net, int batch, const float* r_d, float* z_d);
/* Levels of at most `rows` rows (default 2048) run their V-cycle steps in
 * one block per vector with block barriers; larger levels one grid-wide
 * launch per step. */
afem_status afem_mpnn_set_coarse_rows(afem_mpnn net, int rows);
/* The level-l smoother weights d_l (level_rows[l] floats). */
afem_status afem_mpnn_scalings(afem_mpnn net, int level, float* d_d);
/* Gradient of the mean relative energy norm of the error propagation,
 * ||e - M r||_A^2 / ||e||_A^2 over the batch of (r = A e, e) pairs (grad_d:
 * param_count floats, nullable) and the loss (host, nullable).  Returns once
 * the device work is done (it reads back the GEMMs' error word). */
afem_status afem_mpnn_gradients(afem_mpnn net, int batch, const float* r_d, const float* e_d, float* grad_d,
                                double* loss_h);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) on that loss. */
afem_status afem_mpnn_train_step(afem_mpnn net, int batch, const float* r_d, const float* e_d, float lr,
                                 double* loss_h);
/* The network's layer GEMMs on their own (the tcgen05 kernels; testing and
 * reuse).  Y[M x 64] = act(X1 W1 + X2 W2 + bias): X1, X2 BF16 [M][64]
 * row-major (X2 and W2t null: one product), W given transposed, Wt[n][k]
 * BF16 64 x 64, bias FP32 [64] nullable, relu 0/1; outputs Yb BF16 [M][64]
 * and/or Yf FP32 [M][64] (accumulate: Yf += ...).  Device pointers, 16-byte
 * aligned.  Synchronous. */
afem_status afem_tc_row_gemm(afem_context ctx, int64_t M, const void* X1_d, const void* W1t_d, const void* X2_d,
                             const void* W2t_d, const float* bias_d, int relu, void* Yb_d, float* Yf_d,
                             int accumulate);
/* dW = [X1^T G ; X2^T G] summed over the M rows: FP32 [2][64][64], fixed
 * summation order (deterministic).  Synchronous. */
afem_status afem_tc_weight_grad(afem_context ctx, int64_t M, const void* X1_d, const void* X2_d, const void* G_d,
                                float* dW_d);
/* Flexible CG (FCG(1)) on the FP64 CSR system with M as the preconditioner;
 * FP64 vectors, dots and true residual, M applied in FP32.  Synchronous. */
afem_status afem_fcg_solve(afem_context ctx, int n, const int32_t* row_ptr_d, const int32_t* cols_d,
                           const double* values_d, const double* b_d, double* x_d, afem_mpnn net,
                           const afem_solver_options* opt, afem_solve_info* info);

/* precond = learned of the linear-system service: the network whose
 * level-0 graph is this system's matrix pattern (afem_mpnn_create with the
 * system's row_ptr / cols, on the same context), used by afem_ls_solve when
 * opt->precond = AFEM_PRECOND_LEARNED (NULL detaches it).  The system does
 * not own it.  No reference counterpart (the reference hands the solve to
 * HYPRE / PETSc / Aleph, femutils/HypreDoFLinearSystem.cc:596-751). */
afem_status afem_ls_set_learned_preconditioner(afem_linear_system ls, afem_mpnn net);

/* ---------------------------------------------------------------------- */
/* Batched 2D Poisson P1: many independent instances (the Poisson module's
 * assemble + Dirichlet elimination + solve, modules/poisson/FemModule.cc:
 * 163-196, once per instance) with 4 right-hand sides each, assembled and
 * solved in ONE persistent cooperative launch captured in a CUDA graph.
 * Each instance is solved by its own team of CTAs (sized by a cost model);
 * FP64 iterative refinement around FP32 Jacobi CG.  No counterpart in the
 * reference, which runs one system per module execution. */
typedef struct afem_batch_s* afem_batch;

typedef struct {
  int nb_node, nb_cell;
  const double* coords_d;       /* [nb_node][3] */
  const int32_t* cells_d;       /* [nb_cell][3] triangles */
  const int32_t* nc_ptr_d;      /* node -> cell incidence (afem_node_cell_build) */
  const int32_t* nc_cell_d;
  const uint8_t* nc_local_d;
  const uint8_t* nc_slot_d;     /* slot map (afem_sparsity_cols) */
  const int32_t* row_ptr_d;     /* CSR structure (afem_sparsity_rows / _cols) */
  const int32_t* cols_d;
  const uint8_t* dirichlet_d;   /* [nb_node]: 1 = u = 0 there (row-column elimination) */
  const float* sources_d;       /* [4][8][4]: per right-hand side 8 Gaussian bumps
                                   (amplitude, centre x, centre y, width); f_k(x) =
                                   sum a exp(-|x - c|^2 / (2 w^2)), b_i = m_i f_k(x_i)
                                   with m_i the lumped area (sum of |T| / 3) */
  double* values_d;             /* out: FP64 CSR values after elimination [nnz] */
  double* rhs_d;                /* out: right-hand sides [nb_node][4] */
  double* x_d;                  /* out: solutions [nb_node][4] (16-byte aligned) */
} afem_batch_instance;

typedef struct {
  int block;                    /* threads per CTA: 128, 256 or 512 */
  int blocks_per_sm;            /* CTAs per SM (clamped to the occupancy) */
  float cost_exponent;          /* team size ~ rows^(cost_exponent / 2) */
} afem_batch_config;

typedef struct {
  int inner_iterations;         /* FP32 CG iterations, all refinement steps */
  int refinements;              /* FP64 refinement steps */
  int status;
  float finish_ms;              /* time from the launch's start to this instance's finish */
  double relres[4];             /* final FP64 ||b - A x|| / ||b|| per right-hand side */
} afem_batch_result;

afem_status afem_batch_create(afem_context ctx, int nb_inst, const afem_batch_instance* inst_h, afem_batch* batch);
afem_status afem_batch_destroy(afem_batch batch);
afem_status afem_batch_set_config(afem_batch batch, const afem_batch_config* cfg);
afem_status afem_batch_get_config(afem_batch batch, afem_batch_config* cfg, int* grid);
/* Team sizes in proportion to explicit per-instance weights (nb_inst
 * positive values; null returns to the cost model), e.g. measured
 * finish_ms x CTAs of a previous run. */
afem_status afem_batch_set_weights(afem_batch batch, const double* weights_h);
/* The CTA range of instance `inst` in the persistent grid. */
afem_status afem_batch_team(afem_batch batch, int inst, int* cta0, int* ncta);
/* Assemble and solve every instance (opt: rtol on the FP64 residual,
 * inner_rtol of the FP32 CG, max_iter per inner solve).  results_h: nb_inst
 * entries (nullable); ms: device time of the graph launch (nullable).
 * Synchronous. */
afem_status afem_batch_solve(afem_batch batch, const afem_solver_options* opt, afem_batch_result* results_h,
                             float* ms);
/* Time every candidate configuration (reps timed runs after one warm-up,
 * minimum kept; times_ms[c] = -1 for a candidate that cannot run), keep the
 * fastest (*best = its index). */
afem_status afem_batch_autotune(afem_batch batch, const afem_solver_options* opt, const afem_batch_config* cands,
                                int nb_cands, int reps, float* times_ms, int* best);
/* Failure-detection test: CTA `stall_cta` leaves before its first team
 * barrier, so its teammates' waits run out after `spin_limit` polls and the
 * call returns AFEM_ERR_TIMEOUT with the context still usable. */
afem_status afem_batch_failure_test(afem_batch batch, int stall_cta, long long spin_limit);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif
#endif /* AFEM_GB300_H */
