// Node-wise (atomic-free) P1 assembly.
//
// GB300 issues FP64 at about 1/74 of its FP32 rate (measured ~0.5 T DFMA/s
// against 6.5 TB/s of HBM), so the assembly is bound by FP64 instruction
// count, not by bytes.  The reference recomputes each element once per
// incident node (femutils/BSRFormat.h:406-537: 3x for triangles, 4x for
// tetrahedra); here every element matrix is computed ONCE, in a cell-wise
// kernel with a minimal-operation formulation, and stored as planes
// ke[entry][cell] (structure of arrays, coalesced).  A node-wise kernel then
// sums, for each row, the element rows of its incident cells, in increasing
// cell order, straight into the slots given by the slot map -- no atomics,
// no column search, deterministic.
//
// Element formulation (same quantities as modules/poisson/ElementMatrix.h:41-118
// and femutils/ArcaneFemFunctionsGpu.h:76-128,241-281,414-535, regrouped):
//   tetrahedron: v_k = p_k - p_0, c_1 = v_2 x v_3, c_2 = v_3 x v_1,
//   c_3 = v_1 x v_2, c_0 = -(c_1+c_2+c_3), det = v_1 . c_1 = 6 V (signed);
//   grad N_i = c_i / det, so K_ij = V grad N_i . grad N_j = c_i . c_j / (6|det|).
//   triangle: c_1 = (v_2y, -v_2x), c_2 = (-v_1y, v_1x), c_0 = -(c_1+c_2),
//   A2 = v_1 x v_2; K_ij = c_i . c_j / (2|A2|).
//   Diagonals use the zero row sum of a P1 stiffness: K_ii = -sum_{j!=i} K_ij.
// Results agree with the reference formulas to rounding (tests check 1e-12).
#include <algorithm>

#include "afem_internal.cuh"

namespace afem {

constexpr int kGatherBlock = 128;
constexpr int kScalarRmax = 32;     // scalar row length kept in shared memory
constexpr int kElastRmaxB = 16;     // block row length kept in shared memory (x3 scalars)

struct d3 {
  double x, y, z;
};

__device__ __forceinline__ d3 ld_node(const double* __restrict__ xyz, int32_t n) {
  const double* p = xyz + 3 * (int64_t)n;
  return d3{__ldg(p), __ldg(p + 1), __ldg(p + 2)};
}
__device__ __forceinline__ d3 sub(d3 a, d3 b) { return d3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ d3 cross(d3 a, d3 b) {
  return d3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double dot(d3 a, d3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// packed upper-triangle index of (i, j) in an n x n symmetric matrix
__device__ __forceinline__ int sym_index(int i, int j, int n) {
  int lo = min(i, j), hi = max(i, j);
  return lo * (2 * n - lo + 1) / 2 + (hi - lo);
}

// Tetrahedron geometry: cofactor vectors c[0..3] and s = 1 / (6 |det|).
__device__ __forceinline__ void tet_cofactors(const double* __restrict__ xyz, const int32_t* __restrict__ cn,
                                              int64_t c, d3 cf[4], double* s, double* vol) {
  const int32_t* q = cn + 4 * c;
  int32_t n0 = __ldg(q), n1 = __ldg(q + 1), n2 = __ldg(q + 2), n3 = __ldg(q + 3);
  d3 p0 = ld_node(xyz, n0);
  d3 v1 = sub(ld_node(xyz, n1), p0), v2 = sub(ld_node(xyz, n2), p0), v3 = sub(ld_node(xyz, n3), p0);
  cf[1] = cross(v2, v3);
  cf[2] = cross(v3, v1);
  cf[3] = cross(v1, v2);
  cf[0] = d3{-(cf[1].x + cf[2].x + cf[3].x), -(cf[1].y + cf[2].y + cf[3].y), -(cf[1].z + cf[2].z + cf[3].z)};
  double det = fabs(dot(v1, cf[1]));
  *vol = det / 6.0;
  *s = 1.0 / (6.0 * det);
}

// ---------------------------------------------------------------------------
// Element kernels.

// Poisson tetrahedron: 10 planes (packed upper triangle of the 4x4 matrix).
__global__ void __launch_bounds__(256) k_elem_poisson_tet(int nb_cell, const double* __restrict__ xyz,
                                                          const int32_t* __restrict__ cn,
                                                          const double* __restrict__ coeff, double* __restrict__ ke) {
  const int64_t C = nb_cell;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x) {
    d3 cf[4];
    double s, vol;
    tet_cofactors(xyz, cn, c, cf, &s, &vol);
    if (coeff) s *= __ldg(coeff + c);
    double k01 = s * dot(cf[0], cf[1]), k02 = s * dot(cf[0], cf[2]), k03 = s * dot(cf[0], cf[3]);
    double k12 = s * dot(cf[1], cf[2]), k13 = s * dot(cf[1], cf[3]), k23 = s * dot(cf[2], cf[3]);
    ke[0 * C + c] = -(k01 + k02 + k03);
    ke[1 * C + c] = k01;
    ke[2 * C + c] = k02;
    ke[3 * C + c] = k03;
    ke[4 * C + c] = -(k01 + k12 + k13);
    ke[5 * C + c] = k12;
    ke[6 * C + c] = k13;
    ke[7 * C + c] = -(k02 + k12 + k23);
    ke[8 * C + c] = k23;
    ke[9 * C + c] = -(k03 + k13 + k23);
  }
}

// Poisson triangle: 6 planes.
__global__ void __launch_bounds__(256) k_elem_poisson_tri(int nb_cell, const double* __restrict__ xyz,
                                                          const int32_t* __restrict__ cn,
                                                          const double* __restrict__ coeff, double* __restrict__ ke) {
  const int64_t C = nb_cell;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x) {
    const int32_t* q = cn + 3 * c;
    int32_t n0 = __ldg(q), n1 = __ldg(q + 1), n2 = __ldg(q + 2);
    const double* a0 = xyz + 3 * (int64_t)n0;
    const double* a1 = xyz + 3 * (int64_t)n1;
    const double* a2 = xyz + 3 * (int64_t)n2;
    double x0 = __ldg(a0), y0 = __ldg(a0 + 1);
    double v1x = __ldg(a1) - x0, v1y = __ldg(a1 + 1) - y0;
    double v2x = __ldg(a2) - x0, v2y = __ldg(a2 + 1) - y0;
    double A2 = v1x * v2y - v1y * v2x;
    double s = 1.0 / (2.0 * fabs(A2));
    if (coeff) s *= __ldg(coeff + c);
    // c1 = (v2y, -v2x), c2 = (-v1y, v1x), c0 = -(c1 + c2)
    double c0x = v1y - v2y, c0y = v2x - v1x;
    double k01 = s * (c0x * v2y - c0y * v2x);
    double k02 = s * (c0y * v1x - c0x * v1y);
    double k12 = s * (-(v2y * v1y) - v2x * v1x);
    ke[0 * C + c] = -(k01 + k02);
    ke[1 * C + c] = k01;
    ke[2 * C + c] = k02;
    ke[3 * C + c] = -(k01 + k12);
    ke[4 * C + c] = k12;
    ke[5 * C + c] = -(k02 + k12);
  }
}

// Elasticity tetrahedron: 78 planes = 6 off-diagonal 3x3 blocks (n < m, 9
// each, row-major) followed by 4 diagonal blocks (6 each, packed upper).
// Block (n, m) rows a / columns b:
//   K_ab = V [lambda dN_n/dx_a dN_m/dx_b + mu dN_n/dx_b dN_m/dx_a
//             + mu delta_ab grad N_n . grad N_m]
// which is modules/elasticity/ElementMatrix.h:216-301 (normal strain +
// compressibility + shear) regrouped; diagonal blocks by zero block-row sum.
__global__ void __launch_bounds__(128) k_elem_elasticity_tet(int nb_cell, const double* __restrict__ xyz,
                                                             const int32_t* __restrict__ cn, double lambda, double mu,
                                                             double* __restrict__ ke) {
  const int64_t C = nb_cell;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < C; c += (int64_t)gridDim.x * blockDim.x) {
    d3 cf[4];
    double s, vol;
    tet_cofactors(xyz, cn, c, cf, &s, &vol);
    const double ls = lambda * s, ms = mu * s, lms = (lambda + mu) * s;
    double dg[4][6];
#pragma unroll
    for (int n = 0; n < 4; ++n)
#pragma unroll
      for (int k = 0; k < 6; ++k) dg[n][k] = 0.0;
    int pair = 0;
#pragma unroll
    for (int n = 0; n < 4; ++n) {
#pragma unroll
      for (int m = n + 1; m < 4; ++m) {
        const double cn_[3] = {cf[n].x, cf[n].y, cf[n].z};
        const double cm_[3] = {cf[m].x, cf[m].y, cf[m].z};
        double P[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) P[a][b] = cn_[a] * cm_[b];
        const double msS = ms * (P[0][0] + P[1][1] + P[2][2]);
        double B[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) B[a][b] = (a == b) ? fma(lms, P[a][a], msS) : fma(ls, P[a][b], ms * P[b][a]);
        double* out = ke + (int64_t)(pair * 9) * C + c;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) out[(int64_t)(a * 3 + b) * C] = B[a][b];
        // diagonal blocks: K^nn = -sum_m K^nm, K^mm = -sum_n (K^nm)^T
        int k = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = a; b < 3; ++b, ++k) {
            dg[n][k] -= B[a][b];
            dg[m][k] -= B[b][a];
          }
        ++pair;
      }
    }
#pragma unroll
    for (int n = 0; n < 4; ++n)
#pragma unroll
      for (int k = 0; k < 6; ++k) ke[(int64_t)(54 + n * 6 + k) * C + c] = dg[n][k];
  }
}

// Plane of entry (row node i comp a, column node m comp b) in the 78-plane layout.
__device__ __forceinline__ int elast_plane(int i, int m, int a, int b) {
  if (i == m) {
    int lo = min(a, b), hi = max(a, b);
    return 54 + i * 6 + lo * (5 - lo) / 2 + hi;
  }
  int lo = min(i, m), hi = max(i, m);
  int pair = lo * (7 - lo) / 2 + (hi - lo - 1);
  return pair * 9 + (i < m ? a * 3 + b : b * 3 + a);
}

// ---------------------------------------------------------------------------
// Node-wise gathers.

// One thread per (scalar) row: accumulates the element rows of the incident
// cells in shared memory (row length <= kScalarRmax) or directly in its own
// row of `values` (longer rows), then writes the row.
template <int NPC>
__global__ void __launch_bounds__(kGatherBlock) k_gather_scalar(int nb_node, const int32_t* __restrict__ nc_ptr,
                                                                const int32_t* __restrict__ nc_cell,
                                                                const uint8_t* __restrict__ nc_local,
                                                                const uint8_t* __restrict__ nc_slot,
                                                                const int32_t* __restrict__ row_ptr,
                                                                const double* __restrict__ ke, int nb_cell,
                                                                double* __restrict__ values) {
  __shared__ double acc[kScalarRmax * kGatherBlock];
  const int t = threadIdx.x;
  const int64_t C = nb_cell;
  for (int row = blockIdx.x * blockDim.x + t; row < nb_node; row += gridDim.x * blockDim.x) {
    const int32_t rb = row_ptr[row];
    const int len = row_ptr[row + 1] - rb;
    const bool fast = len <= kScalarRmax;
    if (fast) {
      for (int s = 0; s < len; ++s) acc[s * kGatherBlock + t] = 0.0;
    } else {
      for (int s = 0; s < len; ++s) values[rb + s] = 0.0;
    }
    const int32_t pe = nc_ptr[row + 1];
    for (int32_t p = nc_ptr[row]; p < pe; ++p) {
      const int64_t c = __ldg(nc_cell + p);
      const int i = __ldg(nc_local + p);
      uint8_t sl[NPC];
      if (NPC == 4) {
        uint32_t w = __ldg(reinterpret_cast<const uint32_t*>(nc_slot) + p);
#pragma unroll
        for (int j = 0; j < 4; ++j) sl[j] = (uint8_t)(w >> (8 * j));
      } else {
#pragma unroll
        for (int j = 0; j < NPC; ++j) sl[j] = __ldg(nc_slot + (int64_t)p * NPC + j);
      }
#pragma unroll
      for (int j = 0; j < NPC; ++j) {
        double v = __ldg(ke + (int64_t)sym_index(i, j, NPC) * C + c);
        if (fast)
          acc[sl[j] * kGatherBlock + t] += v;
        else
          values[rb + sl[j]] += v;
      }
    }
    if (fast)
      for (int s = 0; s < len; ++s) values[rb + s] = acc[s * kGatherBlock + t];
  }
}

// One thread per scalar row (node, component a) of the 3x3-block matrix.
__global__ void __launch_bounds__(kGatherBlock) k_gather_elasticity(
    int nb_node, const int32_t* __restrict__ nc_ptr, const int32_t* __restrict__ nc_cell,
    const uint8_t* __restrict__ nc_local, const uint8_t* __restrict__ nc_slot, const int32_t* __restrict__ row_ptr,
    const double* __restrict__ ke, int nb_cell, int per_row_layout, double* __restrict__ values) {
  __shared__ double acc[3 * kElastRmaxB * kGatherBlock];
  const int t = threadIdx.x;
  const int64_t C = nb_cell;
  const int64_t nrow = 3 * (int64_t)nb_node;
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + t; r < nrow; r += (int64_t)gridDim.x * blockDim.x) {
    const int node = (int)(r / 3), a = (int)(r - 3 * (int64_t)node);
    const int32_t rb = row_ptr[node];
    const int len = row_ptr[node + 1] - rb;
    const bool fast = len <= kElastRmaxB;
    // value index of (block x, column comp b) of this scalar row
    auto vidx = [&](int x, int b) -> int64_t {
      return per_row_layout ? (int64_t)rb * 9 + (int64_t)a * 3 * len + 3 * x + b : ((int64_t)rb + x) * 9 + a * 3 + b;
    };
    if (fast) {
      for (int s = 0; s < 3 * len; ++s) acc[s * kGatherBlock + t] = 0.0;
    } else {
      for (int x = 0; x < len; ++x)
        for (int b = 0; b < 3; ++b) values[vidx(x, b)] = 0.0;
    }
    const int32_t pe = nc_ptr[node + 1];
    for (int32_t p = nc_ptr[node]; p < pe; ++p) {
      const int64_t c = __ldg(nc_cell + p);
      const int i = __ldg(nc_local + p);
      const uint32_t w = __ldg(reinterpret_cast<const uint32_t*>(nc_slot) + p);
#pragma unroll
      for (int m = 0; m < 4; ++m) {
        const int x = (w >> (8 * m)) & 0xff;
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          double v = __ldg(ke + (int64_t)elast_plane(i, m, a, b) * C + c);
          if (fast)
            acc[(3 * x + b) * kGatherBlock + t] += v;
          else
            values[vidx(x, b)] += v;
        }
      }
    }
    if (fast)
      for (int x = 0; x < len; ++x)
        for (int b = 0; b < 3; ++b) values[vidx(x, b)] = acc[(3 * x + b) * kGatherBlock + t];
  }
}

// ---------------------------------------------------------------------------
// Right-hand sides.

// w_c = qdot * measure / npc (ArcaneFemFunctionsGpu.h:703: sum += qdot * domain / nbItem)
__global__ void k_cell_source_weight(int nb_cell, int dim, const double* __restrict__ xyz,
                                     const int32_t* __restrict__ cn, double qdot, double* __restrict__ w) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nb_cell; c += (int64_t)gridDim.x * blockDim.x) {
    double meas;
    int npc;
    if (dim == 2) {
      const int32_t* q = cn + 3 * c;
      const double* a0 = xyz + 3 * (int64_t)q[0];
      const double* a1 = xyz + 3 * (int64_t)q[1];
      const double* a2 = xyz + 3 * (int64_t)q[2];
      double v1x = a1[0] - a0[0], v1y = a1[1] - a0[1], v2x = a2[0] - a0[0], v2y = a2[1] - a0[1];
      meas = fabs(v1x * v2y - v1y * v2x) / 2.0;
      npc = 3;
    } else {
      d3 cf[4];
      double s;
      tet_cofactors(xyz, cn, c, cf, &s, &meas);
      npc = 4;
    }
    w[c] = qdot * meas / npc;
  }
}

// rhs[node * stride + off] = sum_{cells, increasing} w_c                 (body = 0)
// rhs[node * stride + off] += sum_{cells, increasing} f * w_c / 4        (body = 1,
//   the += f[k] * volume / 4 of modules/elasticity/BodyForce.h:155-157)
__global__ void k_node_sum(int nb_node, const int32_t* __restrict__ nc_ptr, const int32_t* __restrict__ nc_cell,
                           const double* __restrict__ w, int stride, int off, double f, int body,
                           double* __restrict__ rhs) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nb_node; n += gridDim.x * blockDim.x) {
    int64_t d = (int64_t)n * stride + off;
    double sum = body ? rhs[d] : 0.0;
    for (int32_t p = nc_ptr[n]; p < nc_ptr[n + 1]; ++p) {
      double wc = w[nc_cell[p]];
      sum += body ? f * wc / 4 : wc;
    }
    rhs[d] = sum;
  }
}

__global__ void k_cell_volume(int nb_cell, const double* __restrict__ xyz, const int32_t* __restrict__ cn,
                              double* __restrict__ vol) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nb_cell; c += (int64_t)gridDim.x * blockDim.x) {
    d3 cf[4];
    double s, v;
    tet_cofactors(xyz, cn, c, cf, &s, &v);
    vol[c] = v;
  }
}

static afem_status check_mesh(const afem_mesh_view* m, const char* who) {
  AFEM_CHECK_ARG(m != nullptr, "%s: null mesh view", who);
  AFEM_CHECK_ARG(m->dim == 2 || m->dim == 3, "%s: dim must be 2 or 3 (got %d)", who, m->dim);
  AFEM_CHECK_ARG(m->nb_node > 0 && m->nb_cell > 0, "%s: empty mesh", who);
  AFEM_CHECK_ARG(m->coords_d && m->cell_nodes_d && m->nc_ptr_d && m->nc_cell_d && m->nc_local_d,
                 "%s: null mesh buffer", who);
  return AFEM_OK;
}

}  // namespace afem

using namespace afem;

extern "C" {

afem_status afem_element_matrices_poisson_p1(afem_context ctx, const afem_mesh_view* m, const double* cell_coeff_d,
                                             double* ke) {
  AFEM_CHECK_ARG(ctx, "afem_element_matrices_poisson_p1: null context");
  AFEM_TRY(check_mesh(m, "afem_element_matrices_poisson_p1"));
  AFEM_CHECK_ARG(ke, "afem_element_matrices_poisson_p1: null ke");
  unsigned ge = grid_for(ctx, m->nb_cell, 256, 16);
  if (m->dim == 3)
    return launch(ctx, k_elem_poisson_tet, ge, 256, 0, m->nb_cell, m->coords_d, m->cell_nodes_d, cell_coeff_d, ke);
  return launch(ctx, k_elem_poisson_tri, ge, 256, 0, m->nb_cell, m->coords_d, m->cell_nodes_d, cell_coeff_d, ke);
}

afem_status afem_gather_poisson_p1(afem_context ctx, const afem_mesh_view* m, const int32_t* row_ptr_d,
                                   const double* ke, double* values_d) {
  AFEM_CHECK_ARG(ctx, "afem_gather_poisson_p1: null context");
  AFEM_TRY(check_mesh(m, "afem_gather_poisson_p1"));
  AFEM_CHECK_ARG(m->nc_slot_d && row_ptr_d && ke && values_d, "afem_gather_poisson_p1: null buffer");
  unsigned gg = (unsigned)((m->nb_node + kGatherBlock - 1) / kGatherBlock);
  if (m->dim == 3)
    return launch(ctx, k_gather_scalar<4>, gg, kGatherBlock, 0, m->nb_node, m->nc_ptr_d, m->nc_cell_d, m->nc_local_d,
                  m->nc_slot_d, row_ptr_d, ke, m->nb_cell, values_d);
  return launch(ctx, k_gather_scalar<3>, gg, kGatherBlock, 0, m->nb_node, m->nc_ptr_d, m->nc_cell_d, m->nc_local_d,
                m->nc_slot_d, row_ptr_d, ke, m->nb_cell, values_d);
}

afem_status afem_assemble_poisson_p1(afem_context ctx, const afem_mesh_view* m, const int32_t* row_ptr_d,
                                     const double* cell_coeff_d, double* values_d) {
  AFEM_CHECK_ARG(ctx, "afem_assemble_poisson_p1: null context");
  AFEM_TRY(check_mesh(m, "afem_assemble_poisson_p1"));
  AFEM_CHECK_ARG(m->nc_slot_d && row_ptr_d && values_d, "afem_assemble_poisson_p1: null buffer");
  const int npc = m->dim + 1, nsym = npc * (npc + 1) / 2;
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(double) * (size_t)nsym * m->nb_cell)));
  double* ke;
  AFEM_TRY(scratch_take(ctx, (size_t)nsym * m->nb_cell, &ke));
  AFEM_TRY(afem_element_matrices_poisson_p1(ctx, m, cell_coeff_d, ke));
  return afem_gather_poisson_p1(ctx, m, row_ptr_d, ke, values_d);
}

afem_status afem_element_matrices_elasticity_tet4(afem_context ctx, const afem_mesh_view* m, double lambda,
                                                  double mu, double* ke) {
  AFEM_CHECK_ARG(ctx, "afem_element_matrices_elasticity_tet4: null context");
  AFEM_TRY(check_mesh(m, "afem_element_matrices_elasticity_tet4"));
  AFEM_CHECK_ARG(m->dim == 3, "afem_element_matrices_elasticity_tet4: tetrahedra only (dim 3)");
  AFEM_CHECK_ARG(ke, "afem_element_matrices_elasticity_tet4: null ke");
  return launch(ctx, k_elem_elasticity_tet, grid_for(ctx, m->nb_cell, 128, 16), 128, 0, m->nb_cell, m->coords_d,
                m->cell_nodes_d, lambda, mu, ke);
}

afem_status afem_gather_elasticity_tet4(afem_context ctx, const afem_mesh_view* m, const int32_t* row_ptr_d,
                                        const double* ke, int layout, double* values_d) {
  AFEM_CHECK_ARG(ctx, "afem_gather_elasticity_tet4: null context");
  AFEM_TRY(check_mesh(m, "afem_gather_elasticity_tet4"));
  AFEM_CHECK_ARG(m->dim == 3, "afem_gather_elasticity_tet4: tetrahedra only (dim 3)");
  AFEM_CHECK_ARG(layout == AFEM_LAYOUT_PER_BLOCK || layout == AFEM_LAYOUT_PER_ROW,
                 "afem_gather_elasticity_tet4: bad layout %d", layout);
  AFEM_CHECK_ARG(m->nc_slot_d && row_ptr_d && ke && values_d, "afem_gather_elasticity_tet4: null buffer");
  unsigned gg = (unsigned)((3 * (int64_t)m->nb_node + kGatherBlock - 1) / kGatherBlock);
  return launch(ctx, k_gather_elasticity, gg, kGatherBlock, 0, m->nb_node, m->nc_ptr_d, m->nc_cell_d, m->nc_local_d,
                m->nc_slot_d, row_ptr_d, ke, m->nb_cell, (int)(layout == AFEM_LAYOUT_PER_ROW), values_d);
}

afem_status afem_assemble_elasticity_tet4(afem_context ctx, const afem_mesh_view* m, const int32_t* row_ptr_d,
                                          double lambda, double mu, int layout, double* values_d) {
  AFEM_CHECK_ARG(ctx, "afem_assemble_elasticity_tet4: null context");
  AFEM_TRY(check_mesh(m, "afem_assemble_elasticity_tet4"));
  AFEM_CHECK_ARG(m->nc_slot_d && row_ptr_d && values_d, "afem_assemble_elasticity_tet4: null buffer");
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(double) * (size_t)78 * m->nb_cell)));
  double* ke;
  AFEM_TRY(scratch_take(ctx, (size_t)78 * m->nb_cell, &ke));
  AFEM_TRY(afem_element_matrices_elasticity_tet4(ctx, m, lambda, mu, ke));
  return afem_gather_elasticity_tet4(ctx, m, row_ptr_d, ke, layout, values_d);
}

afem_status afem_rhs_constant_source(afem_context ctx, const afem_mesh_view* m, double qdot, int nb_dof,
                                     double* rhs_d) {
  AFEM_CHECK_ARG(ctx, "afem_rhs_constant_source: null context");
  AFEM_TRY(check_mesh(m, "afem_rhs_constant_source"));
  AFEM_CHECK_ARG(nb_dof >= 1 && rhs_d, "afem_rhs_constant_source: bad nb_dof or null rhs");
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(double) * (size_t)m->nb_cell)));
  double* w;
  AFEM_TRY(scratch_take(ctx, (size_t)m->nb_cell, &w));
  AFEM_TRY(launch(ctx, k_cell_source_weight, grid_for(ctx, m->nb_cell, 256), 256, 0, m->nb_cell, m->dim,
                  m->coords_d, m->cell_nodes_d, qdot, w));
  return launch(ctx, k_node_sum, grid_for(ctx, m->nb_node, 256), 256, 0, m->nb_node, m->nc_ptr_d, m->nc_cell_d,
                (const double*)w, nb_dof, 0, 0.0, 0, rhs_d);
}

afem_status afem_rhs_body_force_tet4(afem_context ctx, const afem_mesh_view* m, double fx, double fy, double fz,
                                     double* rhs_d) {
  AFEM_CHECK_ARG(ctx, "afem_rhs_body_force_tet4: null context");
  AFEM_TRY(check_mesh(m, "afem_rhs_body_force_tet4"));
  AFEM_CHECK_ARG(m->dim == 3 && rhs_d, "afem_rhs_body_force_tet4: tetrahedra only, non-null rhs");
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(double) * (size_t)m->nb_cell)));
  double* vol;
  AFEM_TRY(scratch_take(ctx, (size_t)m->nb_cell, &vol));
  AFEM_TRY(launch(ctx, k_cell_volume, grid_for(ctx, m->nb_cell, 256), 256, 0, m->nb_cell, m->coords_d,
                  m->cell_nodes_d, vol));
  const double f[3] = {fx, fy, fz};
  for (int k = 0; k < 3; ++k) {
    if (f[k] == 0.0) continue;
    AFEM_TRY(launch(ctx, k_node_sum, grid_for(ctx, m->nb_node, 256), 256, 0, m->nb_node, m->nc_ptr_d, m->nc_cell_d,
                    (const double*)vol, 3, k, f[k], 1, rhs_d));
  }
  return AFEM_OK;
}

}  // extern "C"
