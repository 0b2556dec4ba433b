// Node-wise (atomic-free) P1 assembly.
//
// GB300 issues FP64 at about 1/74 of its FP32 rate (measured ~0.5 T DFMA/s
// against 6.5 TB/s of HBM), so the assembly is bound by FP64 instruction
// count, not by bytes.  The reference recomputes each element once per
// incident node (femutils/BSRFormat.h:406-537: 3x for triangles, 4x for
// tetrahedra); here every element matrix is computed ONCE, in a cell-wise
// kernel with a minimal-operation formulation.  Its rows are stored in
// incidence order: row i of cell c goes to the slot of incidence
// p = nc_inverse[c][i] of the node -> cell lists, so that a node-wise kernel
// then STREAMS, for each row, the contiguous element rows of its incident
// cells (in increasing cell order) and adds them into the slots given by the
// slot map -- no atomics, no column search, deterministic.  Each element row
// holds the diagonal entry first, then the other cell nodes in increasing
// local index (the order of the slot map), so that the gather keeps the
// diagonal -- which every incident cell updates -- in a register.
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
#include <atomic>
#include <cmath>
#include <mutex>

#include "afem_elem_ref.cuh"
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

// 32-byte row stores / loads as two 16-byte vector accesses (rows are 32-byte aligned)
__device__ __forceinline__ void st4(double* p, double a, double b, double c, double d) {
  reinterpret_cast<double2*>(p)[0] = make_double2(a, b);
  reinterpret_cast<double2*>(p)[1] = make_double2(c, d);
}
__device__ __forceinline__ void ld4(const double* __restrict__ p, double v[4]) {
  const double2 a = __ldg(reinterpret_cast<const double2*>(p));
  const double2 b = __ldg(reinterpret_cast<const double2*>(p) + 1);
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}

// ---------------------------------------------------------------------------
// Element kernels (one thread per cell).

// AFEM_FORMULATION_MINIMAL.
// Poisson tetrahedron: 4 rows of 4 values, row i at er[inv[c][i] * 4] as
// (K_ii, then K_ij for j != i increasing).  FP64 issue is the binding limit
// on GB300, so the element is computed with few FP64 instructions (72 per
// cell measured: 21 DADD, 28 DFMA, 23 DMUL): with the cofactor vectors
// c_1..c_3 of the edges from node 0 (c_0 = -(c_1 + c_2 + c_3) is never
// formed), the rows sum to zero, so K_0j = -(K_1j + K_2j + K_3j) and K_00 =
// -(K_01 + K_02 + K_03) follow from the 3x3 block; 1 / (6 |det|) is the
// correctly rounded reciprocal __drcp_rn (an FP32 seed with two FP64 Newton
// steps issued more FP64-pipe work: its conversions run there too).
__global__ void __launch_bounds__(256) k_elem_poisson_tet(int cell0, int nb_cell, const double* __restrict__ xyz,
                                                          const int32_t* __restrict__ cn,
                                                          const int32_t* __restrict__ inv,
                                                          const double* __restrict__ coeff, double* __restrict__ er,
                                                          int* __restrict__ bad) {
  for (int64_t c = cell0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nb_cell; c += (int64_t)gridDim.x * blockDim.x) {
    const int4 q = __ldg(reinterpret_cast<const int4*>(cn) + c);
    const d3 p0 = ld_node(xyz, q.x);
    const d3 v1 = sub(ld_node(xyz, q.y), p0), v2 = sub(ld_node(xyz, q.z), p0), v3 = sub(ld_node(xyz, q.w), p0);
    const d3 c1 = cross(v2, v3), c2 = cross(v3, v1), c3 = cross(v1, v2);
    const double v6 = 6.0 * fabs(dot(v1, c1));
    if (bad && !ref::measure_ok(v6)) atomicOr(bad, kFlagDegenerateCell);
    double s = __drcp_rn(v6);
    if (coeff) s *= __ldg(coeff + c);
    const double k11 = s * dot(c1, c1), k22 = s * dot(c2, c2), k33 = s * dot(c3, c3);
    const double k12 = s * dot(c1, c2), k13 = s * dot(c1, c3), k23 = s * dot(c2, c3);
    const double k01 = -(k11 + k12 + k13), k02 = -(k12 + k22 + k23), k03 = -(k13 + k23 + k33);
    const int4 p = __ldg(reinterpret_cast<const int4*>(inv) + c);
    st4(er + 4 * (int64_t)p.x, -(k01 + k02 + k03), k01, k02, k03);
    st4(er + 4 * (int64_t)p.y, k11, k01, k12, k13);
    st4(er + 4 * (int64_t)p.z, k22, k02, k12, k23);
    st4(er + 4 * (int64_t)p.w, k33, k03, k13, k23);
  }
}

// Poisson triangle: 3 rows of 3 values, row i at er[inv[c][i] * 3], diagonal first.
__global__ void __launch_bounds__(256) k_elem_poisson_tri(int cell0, int nb_cell, const double* __restrict__ xyz,
                                                          const int32_t* __restrict__ cn,
                                                          const int32_t* __restrict__ inv,
                                                          const double* __restrict__ coeff, double* __restrict__ er,
                                                          int* __restrict__ bad) {
  for (int64_t c = cell0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nb_cell; c += (int64_t)gridDim.x * blockDim.x) {
    const int32_t* q = cn + 3 * c;
    const double* a0 = xyz + 3 * (int64_t)__ldg(q);
    const double* a1 = xyz + 3 * (int64_t)__ldg(q + 1);
    const double* a2 = xyz + 3 * (int64_t)__ldg(q + 2);
    double x0 = __ldg(a0), y0 = __ldg(a0 + 1);
    double v1x = __ldg(a1) - x0, v1y = __ldg(a1 + 1) - y0;
    double v2x = __ldg(a2) - x0, v2y = __ldg(a2 + 1) - y0;
    double A2 = v1x * v2y - v1y * v2x;
    if (bad && !ref::measure_ok(A2)) atomicOr(bad, kFlagDegenerateCell);
    double s = 1.0 / (2.0 * fabs(A2));
    if (coeff) s *= __ldg(coeff + c);
    // c1 = (v2y, -v2x), c2 = (-v1y, v1x), c0 = -(c1 + c2)
    double c0x = v1y - v2y, c0y = v2x - v1x;
    const double k01 = s * (c0x * v2y - c0y * v2x);
    const double k02 = s * (c0y * v1x - c0x * v1y);
    const double k12 = s * (-(v2y * v1y) - v2x * v1x);
    const int32_t* ip = inv + 3 * c;
    double* r0 = er + 3 * (int64_t)__ldg(ip);
    double* r1 = er + 3 * (int64_t)__ldg(ip + 1);
    double* r2 = er + 3 * (int64_t)__ldg(ip + 2);
    r0[0] = -(k01 + k02); r0[1] = k01; r0[2] = k02;
    r1[0] = -(k01 + k12); r1[1] = k01; r1[2] = k12;
    r2[0] = -(k02 + k12); r2[1] = k02; r2[2] = k12;
  }
}

// AFEM_FORMULATION_REFERENCE / _TESTLAB, Poisson P1 (NPC = 3 triangles, 4
// tetrahedra): the element in the reference's own rounding (afem_elem_ref.cuh).
// Rows are laid out as above (row i at er[inv[c][i] * NPC], diagonal first,
// then the other cell nodes increasing); each row is the reference's element
// vector of its own node, which in the module formulation is not the
// transpose of the column bit for bit ((vol dx_i) dx_k against (vol dx_k) dx_i),
// so every row is formed: 4 x 23 + ~130 FP64 instructions per tetrahedron
// (divisions included) against 72 for the minimal form.  A cell coefficient
// multiplies each entry as the node-wise loop does (coeff * v).
// Which stages of the reference-rounding tetrahedron run their products and
// sums on the integer pipe (afem_fp64_int.cuh) instead of the FP64 pipe, so
// that both pipes work at once: bit 0 the element rows, bit 1 the gradient
// numerators, bit 2 the coordinate differences.  The values are the same bit
// for bit whatever the choice; it is a throughput tuning constant.
#ifndef AFEM_REF_INT_STAGES
#define AFEM_REF_INT_STAGES 0
#endif
constexpr bool kIntRows = (AFEM_REF_INT_STAGES & 1) != 0;
constexpr bool kIntNumerators = (AFEM_REF_INT_STAGES & 2) != 0;
constexpr bool kIntDifferences = (AFEM_REF_INT_STAGES & 4) != 0;

template <int NPC, int F>
__global__ void __launch_bounds__(128) k_elem_poisson_p1_ref(int cell0, int nb_cell, const double* __restrict__ xyz,
                                                             const int32_t* __restrict__ cn,
                                                             const int32_t* __restrict__ inv,
                                                             const double* __restrict__ coeff,
                                                             double* __restrict__ er, int* __restrict__ bad) {
  for (int64_t c = cell0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nb_cell;
       c += (int64_t)gridDim.x * blockDim.x) {
    int32_t nid[NPC], pos[NPC];
    if constexpr (NPC == 4) {
      const int4 q = __ldg(reinterpret_cast<const int4*>(cn) + c);
      const int4 p = __ldg(reinterpret_cast<const int4*>(inv) + c);
      nid[0] = q.x; nid[1] = q.y; nid[2] = q.z; nid[3] = q.w;
      pos[0] = p.x; pos[1] = p.y; pos[2] = p.z; pos[3] = p.w;
    } else {
#pragma unroll
      for (int a = 0; a < NPC; ++a) {
        nid[a] = __ldg(cn + NPC * c + a);
        pos[a] = __ldg(inv + NPC * c + a);
      }
    }
    double n[NPC][3];
#pragma unroll
    for (int a = 0; a < NPC; ++a) {
      const double* p = xyz + 3 * (int64_t)nid[a];
      n[a][0] = __ldg(p);
      n[a][1] = __ldg(p + 1);
      n[a][2] = __ldg(p + 2);
    }
    double K[NPC][NPC], meas;
    if constexpr (F == AFEM_FORMULATION_TESTLAB) {
      if constexpr (NPC == 4) meas = ref::testlab_tet(n, K);
      else meas = ref::testlab_tri(n, K);
#pragma unroll
      for (int i = 0; i < NPC; ++i)
#pragma unroll
        for (int k = 0; k < i; ++k) K[i][k] = K[k][i];
    } else if constexpr (NPC == 4) {
      double g[3][4], vol;
      meas = ref::tet_gradients<kIntDifferences, kIntNumerators>(n, g, &vol);
#pragma unroll
      for (int i = 0; i < 4; ++i) ref::tet_row<kIntRows>(g, vol, i, K[i]);
    } else {
      double dx[3], dy[3], area;
      meas = ref::tri_gradients(n, dx, dy, &area);
#pragma unroll
      for (int i = 0; i < 3; ++i) ref::tri_row(dx, dy, area, i, K[i]);
    }
    if (bad && !ref::measure_ok(meas)) atomicOr(bad, kFlagDegenerateCell);
    if (coeff) {
      const double k = __ldg(coeff + c);
#pragma unroll
      for (int i = 0; i < NPC; ++i)
#pragma unroll
        for (int j = 0; j < NPC; ++j) K[i][j] = ref::mul(k, K[i][j]);
    }
#pragma unroll
    for (int i = 0; i < NPC; ++i) {
      double r[NPC];
      r[0] = K[i][i];
      int q = 1;
#pragma unroll
      for (int j = 0; j < NPC; ++j)
        if (j != i) r[q++] = K[i][j];
      double* dst = er + NPC * (int64_t)pos[i];
      if constexpr (NPC == 4) {
        st4(dst, r[0], r[1], r[2], r[3]);
      } else {
#pragma unroll
        for (int j = 0; j < NPC; ++j) dst[j] = r[j];
      }
    }
  }
}

// Elasticity tetrahedron: for each local node n, its 3x12 row block
// er[inv[c][n] * 36 + a * 12 + 3 q + b], column-node position q = 0 for n
// itself, then the other local nodes in increasing order.  Block (n, m) rows a / columns b:
//   K_ab = V [lambda dN_n/dx_a dN_m/dx_b + mu dN_n/dx_b dN_m/dx_a
//             + mu delta_ab grad N_n . grad N_m]
// which is modules/elasticity/ElementMatrix.h:216-301 (normal strain +
// compressibility + shear) regrouped; diagonal blocks by zero block-row sum.
//
// Each thread computes the 78 distinct values of its cell (6 off-diagonal
// 3x3 blocks, 4 symmetric diagonal blocks) into shared memory; the warp then
// writes the 4 x 32 row blocks (288 B each) with 16-byte stores, 18 lanes per
// row block, so that every written sector is complete.  The packed source
// positions of each 16-byte chunk come from a per-block table, and a lane's
// (cell, chunk) position advances by 32 chunks per pass without a division.
constexpr int kElastElemBlock = 64;
constexpr int kElastPacked = 78;

// packed position of entry (row node i comp a, column node m comp b)
__device__ __forceinline__ int elast_packed(int i, int m, int a, int b) {
  if (i == m) {
    const int lo = min(a, b), hi = max(a, b);
    return 54 + i * 6 + lo * (5 - lo) / 2 + hi;
  }
  const int lo = min(i, m), hi = max(i, m);
  const int pair = lo * (7 - lo) / 2 + (hi - lo - 1);
  return pair * 9 + (i < m ? a * 3 + b : b * 3 + a);
}

// One entry of the reference's elasticity row block (modules/elasticity/
// ElementMatrix.h:216-301) for row component a, column component b, with
// P[x][y] = dN_row/dx_x * dN_col/dx_y: of the reference's twelve-vector sums
// ne + ce + se, every term with a zero factor is an exact zero, which leaves
//   a == b: (l2m P_aa) vol + (mu (P_bb + P_cc)) vol  (b, c the two other axes,
//           summed in the reference's order)
//   a != b: (lambda P_ab) vol + (mu P_ba) vol
// with each product rounded as the reference rounds it.  The products commute,
// so K is symmetric bit for bit.
// INT: 0 all on the FP64 pipe, 1 all on the integer pipe, 2 the mu (shear)
// terms and the final sum on the integer pipe, the rest on the FP64 pipe.
template <int INT>
__device__ __forceinline__ double elast_ref_entry(int a, int b, const double P[3][3], double l2m, double lambda,
                                                  double mu, double vol) {
  auto add1 = [](double x, double y) { return ref::xadd<INT == 1>(x, y); };
  auto mul1 = [](double x, double y) { return ref::xmul<INT == 1>(x, y); };
  auto add2 = [](double x, double y) { return ref::xadd<INT != 0>(x, y); };
  auto mul2 = [](double x, double y) { return ref::xmul<INT != 0>(x, y); };
  if (a == b) {
    const double z = a == 0 ? add2(P[1][1], P[2][2]) : (a == 1 ? add2(P[0][0], P[2][2]) : add2(P[1][1], P[0][0]));
    return add2(mul1(mul1(l2m, P[a][a]), vol), mul2(mul2(mu, z), vol));
  }
  return add2(mul1(mul1(lambda, P[a][b]), vol), mul2(mul2(mu, P[b][a]), vol));
}

// Integer-pipe stages of the reference-rounding elasticity element (as
// AFEM_REF_INT_STAGES for the Poisson tetrahedron): bit 0 the block entries,
// bit 1 the gradient products P, bit 2 the gradient numerators, bit 3 only
// the shear terms of the block entries (when bit 0 is clear).
#ifndef AFEM_ELAST_INT_STAGES
#define AFEM_ELAST_INT_STAGES 0
#endif
constexpr int kElastIntEntries = (AFEM_ELAST_INT_STAGES & 1) ? 1 : ((AFEM_ELAST_INT_STAGES & 8) ? 2 : 0);
constexpr bool kElastIntProducts = (AFEM_ELAST_INT_STAGES & 2) != 0;
constexpr bool kElastIntNumerators = (AFEM_ELAST_INT_STAGES & 4) != 0;

template <int F>
__global__ void __launch_bounds__(kElastElemBlock) k_elem_elasticity_tet(int cell0, int nb_cell, const double* __restrict__ xyz,
                                                                         const int32_t* __restrict__ cn,
                                                                         const int32_t* __restrict__ inv,
                                                                         double lambda, double mu,
                                                                         double* __restrict__ er, int* __restrict__ bad) {
  __shared__ double stage[kElastElemBlock][kElastPacked + 1];
  __shared__ int4 stage_p[kElastElemBlock];
  // src_tab[n][q]: packed positions of entries 2q and 2q + 1 of node n's row block
  __shared__ uint32_t src_tab[4][18];
  for (int i = threadIdx.x; i < 72; i += blockDim.x) {
    const int n = i / 18, q = i - 18 * n;
    uint32_t two = 0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      // row-block position pos = a * 12 + 3 * qn + b: column-node position qn is
      // 0 for the row's own node n, then the other local nodes increasing
      const int pos = 2 * q + h, a = pos / 12, rem = pos - 12 * a, qn = rem / 3, bb = rem - 3 * qn;
      const int m = qn == 0 ? n : qn - 1 + (qn - 1 >= n);
      two |= (uint32_t)elast_packed(n, m, a, bb) << (16 * h);
    }
    src_tab[n][q] = two;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wbase = threadIdx.x & ~31;
  for (int64_t base = cell0 + blockIdx.x * (int64_t)blockDim.x; base < nb_cell; base += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = base + threadIdx.x;
    double* my = stage[threadIdx.x];
    if (c < nb_cell && F != AFEM_FORMULATION_MINIMAL) {
      // reference rounding: gradients and volume of the reference, then the 78
      // distinct entries (6 node-pair blocks, 4 symmetric diagonal blocks)
      const int4 q = __ldg(reinterpret_cast<const int4*>(cn) + c);
      const int32_t nid[4] = {q.x, q.y, q.z, q.w};
      double n[4][3];
#pragma unroll
      for (int a = 0; a < 4; ++a) {
        const double* p = xyz + 3 * (int64_t)nid[a];
        n[a][0] = __ldg(p);
        n[a][1] = __ldg(p + 1);
        n[a][2] = __ldg(p + 2);
      }
      double g[3][4], vol;
      const double v6 = ref::tet_gradients<false, kElastIntNumerators>(n, g, &vol);
      if (bad && !ref::measure_ok(v6)) atomicOr(bad, kFlagDegenerateCell);
      stage_p[threadIdx.x] = __ldg(reinterpret_cast<const int4*>(inv) + c);
      const double l2m = ref::add(lambda, 2.0 * mu);
#pragma unroll
      for (int lo = 0; lo < 4; ++lo)
#pragma unroll
        for (int hi = lo + 1; hi < 4; ++hi) {
          const int pair = lo * (7 - lo) / 2 + (hi - lo - 1);
          double P[3][3];
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) P[a][b] = ref::xmul<kElastIntProducts>(g[a][lo], g[b][hi]);
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
              my[pair * 9 + a * 3 + b] = elast_ref_entry<kElastIntEntries>(a, b, P, l2m, lambda, mu, vol);
        }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        double P[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = a; b < 3; ++b) P[a][b] = P[b][a] = ref::xmul<kElastIntProducts>(g[a][i], g[b][i]);
        int k = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = a; b < 3; ++b, ++k)
            my[54 + i * 6 + k] = elast_ref_entry<kElastIntEntries>(a, b, P, l2m, lambda, mu, vol);
      }
    } else if (c < nb_cell) {
      // cofactors c_1..c_3 of the edges from node 0 and s = 1 / (6 |det|);
      // with G_n = s c_n the block of nodes (n, m) is
      //   K_nm = lambda G_n G_m^T + mu G_m G_n^T + mu (G_n . G_m) I  (times 6 |det| s = 1 here)
      // computed directly for 1 <= n <= m <= 3; the blocks of node 0 follow from the
      // zero column sums (rigid translations): K_0m = -(K_1m + K_2m + K_3m), K_00 = -sum_m K_0m
      const int4 q = __ldg(reinterpret_cast<const int4*>(cn) + c);
      const d3 p0 = ld_node(xyz, q.x);
      const d3 v1 = sub(ld_node(xyz, q.y), p0), v2 = sub(ld_node(xyz, q.z), p0), v3 = sub(ld_node(xyz, q.w), p0);
      const d3 c1 = cross(v2, v3), c2 = cross(v3, v1), c3 = cross(v1, v2);
      const double v6 = 6.0 * fabs(dot(v1, c1));
      if (bad && !ref::measure_ok(v6)) atomicOr(bad, kFlagDegenerateCell);
      const double s = __drcp_rn(v6);
      const double ls = lambda * s, ms = mu * s, lms = (lambda + mu) * s;
      stage_p[threadIdx.x] = __ldg(reinterpret_cast<const int4*>(inv) + c);
      const double cv[3][3] = {{c1.x, c1.y, c1.z}, {c2.x, c2.y, c2.z}, {c3.x, c3.y, c3.z}};
      // K0[m] accumulates K_0,m+1 = -(sum over n = 1..3 of K_n,m+1); it starts as -K_m+1,m+1
      double K0[3][3][3];
#pragma unroll
      for (int n = 0; n < 3; ++n) {   // diagonal blocks of nodes 1..3: (lambda + mu) c c^T + mu |c|^2 I
        double P[3][3];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = a; b < 3; ++b) P[a][b] = cv[n][a] * cv[n][b];
        const double msS = ms * (P[0][0] + P[1][1] + P[2][2]);
        int k = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = a; b < 3; ++b, ++k) {
            const double v = a == b ? fma(lms, P[a][a], msS) : lms * P[a][b];
            my[54 + (n + 1) * 6 + k] = v;
            K0[n][a][b] = -v;
            K0[n][b][a] = -v;
          }
      }
      int pair = 3;
#pragma unroll
      for (int n = 0; n < 3; ++n)   // off-diagonal blocks of nodes 1..3, pairs (1,2) (1,3) (2,3)
#pragma unroll
        for (int m = n + 1; m < 3; ++m, ++pair) {
          double Q[3][3];
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) Q[a][b] = cv[n][a] * cv[m][b];
          const double mS = ms * (Q[0][0] + Q[1][1] + Q[2][2]);
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) {
              const double v = (a == b) ? fma(lms, Q[a][a], mS) : fma(ls, Q[a][b], ms * Q[b][a]);
              my[pair * 9 + a * 3 + b] = v;
              K0[m][a][b] -= v;   // K_nm is in column block m
              K0[n][b][a] -= v;   // K_mn = K_nm^T is in column block n
            }
        }
#pragma unroll
      for (int m = 0; m < 3; ++m)   // pairs (0,1) (0,2) (0,3)
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
          for (int b = 0; b < 3; ++b) my[m * 9 + a * 3 + b] = K0[m][a][b];
      {
        int k = 0;
#pragma unroll
        for (int a = 0; a < 3; ++a)   // K_00 = -(K_01 + K_02 + K_03), upper triangle
#pragma unroll
          for (int b = a; b < 3; ++b, ++k) my[54 + k] = -(K0[0][a][b] + K0[1][a][b] + K0[2][a][b]);
      }
    }
    __syncwarp();
    const int64_t wfirst = base + wbase;
    const int wcount = wfirst < nb_cell ? (int)(nb_cell - wfirst < 32 ? nb_cell - wfirst : 32) : 0;
    // chunk k = 18 t + q of the warp's cells: lane k starts at t = k / 18 and
    // every pass adds 32 = 18 + 14 chunks
    int t = lane >= 18, q = lane - 18 * (lane >= 18);
    for (int k = lane; k < wcount * 18; k += 32) {
      const double* src = stage[wbase + t];
      const int4 p4 = stage_p[wbase + t];
      const int pr[4] = {p4.x, p4.y, p4.z, p4.w};
#pragma unroll
      for (int n = 0; n < 4; ++n) {
        const uint32_t two = src_tab[n][q];
        double* dst = er + 36 * (int64_t)pr[n] + 2 * q;
        *reinterpret_cast<double2*>(dst) = make_double2(src[two & 0xffffu], src[two >> 16]);
      }
      q += 14;
      t += 1 + (q >= 18);
      q -= 18 * (q >= 18);
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Pipelined assembly (afem_assemble_to_host): the first node whose last
// incident cell (the last entry of its ascending incidence list) is at or
// after each cell bound, so that nodes [0, first[k]) are complete once the
// cells below bound[k] are.  Warp minimum, one atomic per warp and bound.
constexpr int kMaxAsmChunks = 16;
struct CellBounds {
  int32_t b[kMaxAsmChunks + 1];
};

// With `need` (nullable): need[k] = the last node whose first incident cell
// (the head of its ascending list) lies below bound[k], so that the cells
// below bound[k] use only nodes [0, need[k]] (warp maximum, one atomic per
// warp and bound; -1 when there is none).
__global__ void k_node_bounds(int nb_node, const int32_t* __restrict__ nc_ptr, const int32_t* __restrict__ nc_cell,
                              int nbound, CellBounds cb, int32_t* __restrict__ first, int32_t* __restrict__ need) {
  const int lane = threadIdx.x & 31;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nr = ((int64_t)nb_node + stride - 1) / stride * stride;   // whole warps in every pass
  for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < nr; n += stride) {
    int32_t last = -1, head = INT_MAX;
    if (n < nb_node) {
      const int32_t b = __ldg(nc_ptr + n), e = __ldg(nc_ptr + n + 1);
      if (e > b) {
        last = __ldg(nc_cell + e - 1);
        head = __ldg(nc_cell + b);
      }
    }
    for (int k = 0; k < nbound; ++k) {
      const int32_t v = (n < nb_node && last >= cb.b[k]) ? (int32_t)n : INT_MAX;
      const int32_t m = __reduce_min_sync(0xffffffffu, v);
      if (lane == 0 && m != INT_MAX) atomicMin(first + k, m);
      if (need) {
        const int32_t u = (n < nb_node && head < cb.b[k]) ? (int32_t)n : -1;
        const int32_t mx = __reduce_max_sync(0xffffffffu, u);
        if (lane == 0 && mx >= 0) atomicMax(need + k, mx);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Node-wise gathers: one thread per (scalar) row streams its contiguous
// element rows and adds them into shared-memory accumulators (row length
// <= kScalarRmax) or directly into its own row of `values` (longer rows).
// The columns of one incidence are distinct nodes of one cell, hence distinct
// accumulator slots: each incidence loads all of its accumulators, adds, then
// stores them, so its read-modify-writes overlap instead of queuing behind
// one another (the compiler cannot prove the slots distinct by itself).  Every
// accumulator still receives its terms in increasing incidence order.

template <int NPC>
__global__ void __launch_bounds__(kGatherBlock) k_gather_scalar(int row0, int nb_node,
                                                                const int32_t* __restrict__ nc_ptr,
                                                                const uint8_t* __restrict__ nc_slot,
                                                                const int32_t* __restrict__ row_ptr,
                                                                const double* __restrict__ er,
                                                                double* __restrict__ values) {
  __shared__ double acc[kScalarRmax * kGatherBlock];
  double* const my = acc + threadIdx.x;   // this thread's accumulators, stride kGatherBlock
  for (int row = row0 + blockIdx.x * blockDim.x + threadIdx.x; row < nb_node; row += gridDim.x * blockDim.x) {
    const int32_t rb = __ldg(row_ptr + row);
    const int len = __ldg(row_ptr + row + 1) - rb;
    const int32_t p0 = __ldg(nc_ptr + row), p1 = __ldg(nc_ptr + row + 1);
    if (len <= kScalarRmax) {
      for (int s = 0; s < len; ++s) my[s * kGatherBlock] = 0.0;
      // the diagonal (first value and slot byte of every incidence) in a register
      double diag = 0.0;
      if constexpr (NPC == 4) {
        const double2* src = reinterpret_cast<const double2*>(er) + 2 * (int64_t)p0;
        const uint32_t* sp = reinterpret_cast<const uint32_t*>(nc_slot) + p0;
#pragma unroll 2
        for (int32_t p = p0; p < p1; ++p, src += 2, ++sp) {
          const double2 a = __ldg(src), b = __ldg(src + 1);
          const uint32_t w = __ldg(sp);
          diag += a.x;
          double* const d1 = my + ((w >> 8) & 0xffu) * kGatherBlock;
          double* const d2 = my + ((w >> 16) & 0xffu) * kGatherBlock;
          double* const d3 = my + (w >> 24) * kGatherBlock;
          const double o1 = *d1, o2 = *d2, o3 = *d3;
          *d1 = o1 + a.y;
          *d2 = o2 + b.x;
          *d3 = o3 + b.y;
        }
      } else {
        const double* src = er + (int64_t)NPC * p0;
        const uint8_t* sp = nc_slot + (int64_t)NPC * p0;
#pragma unroll 2
        for (int32_t p = p0; p < p1; ++p, src += NPC, sp += NPC) {
          diag += __ldg(src);
          double* d[NPC];
          double o[NPC];
#pragma unroll
          for (int j = 1; j < NPC; ++j) d[j] = my + __ldg(sp + j) * kGatherBlock;
#pragma unroll
          for (int j = 1; j < NPC; ++j) o[j] = *d[j];
#pragma unroll
          for (int j = 1; j < NPC; ++j) *d[j] = o[j] + __ldg(src + j);
        }
      }
      if (p1 > p0) my[__ldg(nc_slot + (int64_t)NPC * p0) * kGatherBlock] = diag;
      for (int s = 0; s < len; ++s) values[rb + s] = my[s * kGatherBlock];
    } else {
      // long row: accumulate in this thread's own row of values
      for (int s = 0; s < len; ++s) values[rb + s] = 0.0;
      for (int32_t p = p0; p < p1; ++p)
#pragma unroll
        for (int j = 0; j < NPC; ++j) values[rb + __ldg(nc_slot + (int64_t)NPC * p + j)] += __ldg(er + (int64_t)NPC * p + j);
    }
  }
}

// One thread per scalar row (node, component a) of the 3x3-block matrix.
__global__ void __launch_bounds__(kGatherBlock) k_gather_elasticity(int node0, int nb_node,
                                                                    const int32_t* __restrict__ nc_ptr,
                                                                    const uint8_t* __restrict__ nc_slot,
                                                                    const int32_t* __restrict__ row_ptr,
                                                                    const double* __restrict__ er, int per_row_layout,
                                                                    double* __restrict__ values) {
  __shared__ double acc[3 * kElastRmaxB * kGatherBlock];
  double* const my = acc + threadIdx.x;
  const int64_t nrow = 3 * (int64_t)nb_node;
  for (int64_t r = 3 * (int64_t)node0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrow;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int node = (int)(r / 3), a = (int)(r - 3 * (int64_t)node);
    const int32_t rb = __ldg(row_ptr + node);
    const int len = __ldg(row_ptr + node + 1) - rb;
    const int32_t p0 = __ldg(nc_ptr + node), p1 = __ldg(nc_ptr + node + 1);
    // value index of (block x, column comp b) of this scalar row
    const int64_t row_base = per_row_layout ? (int64_t)rb * 9 + (int64_t)a * 3 * len : (int64_t)rb * 9 + a * 3;
    const int xstride = per_row_layout ? 3 : 9;
    if (len <= kElastRmaxB) {
      for (int s = 0; s < 3 * len; ++s) my[s * kGatherBlock] = 0.0;
      const double2* src = reinterpret_cast<const double2*>(er + 36 * (int64_t)p0 + 12 * a);
      const uint32_t* sp = reinterpret_cast<const uint32_t*>(nc_slot) + p0;
      double self0 = 0.0, self1 = 0.0, self2 = 0.0;   // the row's own 3x3 block, in registers
      for (int32_t p = p0; p < p1; ++p, src += 18, ++sp) {
        const uint32_t w = __ldg(sp);
        double v[12];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          const double2 q = __ldg(src + k);
          v[2 * k] = q.x;
          v[2 * k + 1] = q.y;
        }
        self0 += v[0];
        self1 += v[1];
        self2 += v[2];
        double* d[4];
        double o[12];
#pragma unroll
        for (int m = 1; m < 4; ++m) d[m] = my + 3 * ((w >> (8 * m)) & 0xffu) * kGatherBlock;
#pragma unroll
        for (int m = 1; m < 4; ++m)
#pragma unroll
          for (int b = 0; b < 3; ++b) o[3 * m + b] = d[m][b * kGatherBlock];
#pragma unroll
        for (int m = 1; m < 4; ++m)
#pragma unroll
          for (int b = 0; b < 3; ++b) d[m][b * kGatherBlock] = o[3 * m + b] + v[3 * m + b];
      }
      if (p1 > p0) {
        double* d = my + 3 * (__ldg(nc_slot + 4 * (int64_t)p0) & 0xffu) * kGatherBlock;
        d[0] = self0;
        d[kGatherBlock] = self1;
        d[2 * kGatherBlock] = self2;
      }
      for (int x = 0; x < len; ++x)
#pragma unroll
        for (int b = 0; b < 3; ++b) values[row_base + (int64_t)xstride * x + b] = my[(3 * x + b) * kGatherBlock];
    } else {
      for (int x = 0; x < len; ++x)
        for (int b = 0; b < 3; ++b) values[row_base + (int64_t)xstride * x + b] = 0.0;
      for (int32_t p = p0; p < p1; ++p) {
        const uint32_t w = __ldg(reinterpret_cast<const uint32_t*>(nc_slot) + p);
        const double* src = er + 36 * (int64_t)p + 12 * a;
        for (int m = 0; m < 4; ++m) {
          const int x = (w >> (8 * m)) & 0xff;
          for (int b = 0; b < 3; ++b) values[row_base + (int64_t)xstride * x + b] += __ldg(src + 3 * m + b);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Right-hand sides.

// w_c = qdot * measure / npc (ArcaneFemFunctionsGpu.h:703: sum += qdot * domain / nbItem)
// ---------------------------------------------------------------------------
// Bilinear / trilinear Lagrange elements (Quad4, Hexa8), 2 x 2 (x 2) Gauss
// points: _computeElementVectorQuad4Gpu / _computeElementVectorHexa8Gpu
// (modules/poisson/ElementMatrixHexQuad.h:63-91,239-266) with the Jacobian of
// _computeQuadGradientsAndJacobian / _computeHexaGradientsAndJacobian
// (femutils/ArcaneFemFunctionsGpu.h:298-350,554-586) and the reference
// gradients of femutils/ShapeFunctions.h:123-129,314-345.  The element
// matrix is computed once per cell (the reference recomputes it for each of
// the 4 / 8 incident nodes); row a goes to incidence inv[c][a], diagonal
// first, then the other nodes in increasing local index.

constexpr double kGauss = 0.57735026918962576451;   // 1 / sqrt(3)

template <int N>
__device__ __forceinline__ void write_rows_q1(const double (&K)[N][N], const int32_t* ip, double* er) {
#pragma unroll
  for (int a = 0; a < N; ++a) {
    double* r = er + (int64_t)N * __ldg(ip + a);
    r[0] = K[a][a];
    int q = 1;
#pragma unroll
    for (int b = 0; b < N; ++b)
      if (b != a) r[q++] = K[a < b ? a : b][a < b ? b : a];
  }
}

// Reference-rounding derivative tables (compile-time, the reference's expressions).
__constant__ ref::QuadDN kQuadDnRef = ref::make_quad_dn();
__constant__ ref::HexDN kHexDnRef = ref::make_hex_dn();

template <int N>
__device__ __forceinline__ void scale_upper(double (&K)[N][N], double k) {
#pragma unroll
  for (int a = 0; a < N; ++a)
#pragma unroll
    for (int b = a; b < N; ++b) K[a][b] = ref::mul(k, K[a][b]);
}

// F = AFEM_FORMULATION_MINIMAL: the fewest FP64 instructions (below);
// otherwise the reference's own rounding (ref::quad4_matrix / hexa8_matrix).
template <int F>
__global__ void __launch_bounds__(128) k_elem_poisson_quad4(int cell0, int nb_cell, const double* __restrict__ xyz,
                                                            const int32_t* __restrict__ cn,
                                                            const int32_t* __restrict__ inv,
                                                            const double* __restrict__ coeff, double* __restrict__ er,
                                                            int* __restrict__ bad) {
  for (int64_t c = cell0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nb_cell;
       c += (int64_t)gridDim.x * blockDim.x) {
    double x[4], y[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const double* p = xyz + 3 * (int64_t)__ldg(cn + 4 * c + a);
      x[a] = __ldg(p);
      y[a] = __ldg(p + 1);
    }
    double K[4][4];
    if constexpr (F != AFEM_FORMULATION_MINIMAL) {
      const bool ok = ref::quad4_matrix(x, y, kQuadDnRef, K);
      if (bad && !ok) atomicOr(bad, kFlagDegenerateCell);
      if (coeff) scale_upper<4>(K, __ldg(coeff + c));
      write_rows_q1<4>(K, inv + 4 * c, er);
    } else {
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) K[a][b] = 0.0;
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        const double xi = (g >> 1) ? kGauss : -kGauss, eta = (g & 1) ? kGauss : -kGauss;
        const double dxi[4] = {-0.25 * (1.0 - eta), 0.25 * (1.0 - eta), 0.25 * (1.0 + eta), -0.25 * (1.0 + eta)};
        const double deta[4] = {-0.25 * (1.0 - xi), -0.25 * (1.0 + xi), 0.25 * (1.0 + xi), 0.25 * (1.0 - xi)};
        double j00 = 0.0, j01 = 0.0, j10 = 0.0, j11 = 0.0;
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          j00 += dxi[a] * x[a];
          j01 += dxi[a] * y[a];
          j10 += deta[a] * x[a];
          j11 += deta[a] * y[a];
        }
        const double det = j00 * j11 - j01 * j10;
        if (bad && !ref::measure_ok(det)) atomicOr(bad, kFlagDegenerateCell);
        const double i00 = j11 / det, i01 = -j01 / det, i10 = -j10 / det, i11 = j00 / det;
        double dx[4], dy[4];
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          dx[a] = i00 * dxi[a] + i01 * deta[a];
          dy[a] = i10 * dxi[a] + i11 * deta[a];
        }
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = a; b < 4; ++b) K[a][b] += (dx[a] * dx[b]) * det + (dy[a] * dy[b]) * det;
      }
      if (coeff) {
        const double k = __ldg(coeff + c);
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
          for (int b = a; b < 4; ++b) K[a][b] *= k;
      }
      write_rows_q1<4>(K, inv + 4 * c, er);
    }
  }
}

// Trilinear shape-function derivatives (d/dxi, d/deta, d/dzeta of N_0..N_7) at
// the 2x2x2 Gauss points g = 4 i + 2 j + k, (xi, eta, zeta) = (+-1/sqrt 3)
// with sign (i, j, k): each is +-0.125 (1 +- g)(1 +- g'), three magnitudes,
// written exactly as the double products 0.125 * (1 + g) * (1 + g) etc. round.
constexpr double kHpp = 0.3110042339640731;     // 0.125 (1 + 1/sqrt3)^2
constexpr double kHpm = 0.08333333333333334;    // 0.125 (1 + 1/sqrt3)(1 - 1/sqrt3) = 1/12
constexpr double kHmm = 0.022329099369260228;   // 0.125 (1 - 1/sqrt3)^2
__constant__ double kHexDN[8][3][8] = {
    {{-kHpp, kHpp, kHpm, -kHpm, -kHpm, kHpm, kHmm, -kHmm}, {-kHpp, -kHpm, kHpm, kHpp, -kHpm, -kHmm, kHmm, kHpm}, {-kHpp, -kHpm, -kHmm, -kHpm, kHpp, kHpm, kHmm, kHpm}},
    {{-kHpm, kHpm, kHmm, -kHmm, -kHpp, kHpp, kHpm, -kHpm}, {-kHpm, -kHmm, kHmm, kHpm, -kHpp, -kHpm, kHpm, kHpp}, {-kHpp, -kHpm, -kHmm, -kHpm, kHpp, kHpm, kHmm, kHpm}},
    {{-kHpm, kHpm, kHpp, -kHpp, -kHmm, kHmm, kHpm, -kHpm}, {-kHpp, -kHpm, kHpm, kHpp, -kHpm, -kHmm, kHmm, kHpm}, {-kHpm, -kHmm, -kHpm, -kHpp, kHpm, kHmm, kHpm, kHpp}},
    {{-kHmm, kHmm, kHpm, -kHpm, -kHpm, kHpm, kHpp, -kHpp}, {-kHpm, -kHmm, kHmm, kHpm, -kHpp, -kHpm, kHpm, kHpp}, {-kHpm, -kHmm, -kHpm, -kHpp, kHpm, kHmm, kHpm, kHpp}},
    {{-kHpp, kHpp, kHpm, -kHpm, -kHpm, kHpm, kHmm, -kHmm}, {-kHpm, -kHpp, kHpp, kHpm, -kHmm, -kHpm, kHpm, kHmm}, {-kHpm, -kHpp, -kHpm, -kHmm, kHpm, kHpp, kHpm, kHmm}},
    {{-kHpm, kHpm, kHmm, -kHmm, -kHpp, kHpp, kHpm, -kHpm}, {-kHmm, -kHpm, kHpm, kHmm, -kHpm, -kHpp, kHpp, kHpm}, {-kHpm, -kHpp, -kHpm, -kHmm, kHpm, kHpp, kHpm, kHmm}},
    {{-kHpm, kHpm, kHpp, -kHpp, -kHmm, kHmm, kHpm, -kHpm}, {-kHpm, -kHpp, kHpp, kHpm, -kHmm, -kHpm, kHpm, kHmm}, {-kHmm, -kHpm, -kHpp, -kHpm, kHmm, kHpm, kHpp, kHpm}},
    {{-kHmm, kHmm, kHpm, -kHpm, -kHpm, kHpm, kHpp, -kHpp}, {-kHmm, -kHpm, kHpm, kHmm, -kHpm, -kHpp, kHpp, kHpm}, {-kHmm, -kHpm, -kHpp, -kHpm, kHmm, kHpm, kHpp, kHpm}}};

// Integer-pipe stages of the reference-rounding Hexa8 element: bit 0 the
// matrix accumulation, bit 1 the Jacobians.
#ifndef AFEM_HEX_INT_STAGES
#define AFEM_HEX_INT_STAGES 0
#endif
constexpr bool kHexIntRows = (AFEM_HEX_INT_STAGES & 1) != 0;
constexpr bool kHexIntJacobian = (AFEM_HEX_INT_STAGES & 2) != 0;

template <int F>
__global__ void __launch_bounds__(128) k_elem_poisson_hexa8(int cell0, int nb_cell, const double* __restrict__ xyz,
                                                            const int32_t* __restrict__ cn,
                                                            const int32_t* __restrict__ inv,
                                                            const double* __restrict__ coeff, double* __restrict__ er,
                                                            int* __restrict__ bad) {
  for (int64_t c = cell0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nb_cell;
       c += (int64_t)gridDim.x * blockDim.x) {
    double x[8], y[8], z[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const double* p = xyz + 3 * (int64_t)__ldg(cn + 8 * c + a);
      x[a] = __ldg(p);
      y[a] = __ldg(p + 1);
      z[a] = __ldg(p + 2);
    }
    double K[8][8];
    if constexpr (F != AFEM_FORMULATION_MINIMAL) {
      const bool ok = ref::hexa8_matrix<kHexIntJacobian, kHexIntRows>(x, y, z, kHexDnRef, K);
      if (bad && !ok) atomicOr(bad, kFlagDegenerateCell);
      if (coeff) scale_upper<8>(K, __ldg(coeff + c));
      write_rows_q1<8>(K, inv + 8 * c, er);
    } else {
#pragma unroll
      for (int a = 0; a < 8; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) K[a][b] = 0.0;
      // The trilinear map's derivatives are bilinear in the other two reference
      // coordinates: d x / d xi = m_xi + eta m_xieta + zeta m_xizeta + eta zeta m_xietazeta,
      // and so on, with the moments m (signed sums of the 8 nodal coordinates, / 8)
      // formed once per cell by a Walsh-Hadamard butterfly: 3 FMAs per Jacobian
      // entry per Gauss point instead of 8.  Node a has reference signs
      // (s_xi, s_eta, s_zeta) = (-,-,-) (+,-,-) (+,+,-) (-,+,-) (-,-,+) (+,-,+) (+,+,+) (-,+,+).
      double mo[3][8];   // per component: [1, xi, eta, xi eta, zeta, xi zeta, eta zeta, xi eta zeta]
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const double* v = q == 0 ? x : (q == 1 ? y : z);
        // reorder to the binary order (xi bit 0, eta bit 1, zeta bit 2): nodes 0 1 3 2 4 5 7 6
        const double u0 = v[0], u1 = v[1], u2 = v[3], u3 = v[2], u4 = v[4], u5 = v[5], u6 = v[7], u7 = v[6];
        // stage xi
        const double a0 = u1 + u0, a1 = u1 - u0, a2 = u3 + u2, a3 = u3 - u2;
        const double a4 = u5 + u4, a5 = u5 - u4, a6 = u7 + u6, a7 = u7 - u6;
        // stage eta
        const double b0 = a2 + a0, b1 = a3 + a1, b2 = a2 - a0, b3 = a3 - a1;
        const double b4 = a6 + a4, b5 = a7 + a5, b6 = a6 - a4, b7 = a7 - a5;
        // stage zeta
        mo[q][0] = 0.125 * (b4 + b0);
        mo[q][1] = 0.125 * (b5 + b1);
        mo[q][2] = 0.125 * (b6 + b2);
        mo[q][3] = 0.125 * (b7 + b3);
        mo[q][4] = 0.125 * (b4 - b0);
        mo[q][5] = 0.125 * (b5 - b1);
        mo[q][6] = 0.125 * (b6 - b2);
        mo[q][7] = 0.125 * (b7 - b3);
      }
#pragma unroll 1
      for (int g = 0; g < 8; ++g) {
        const double* dxi = kHexDN[g][0];
        const double* deta = kHexDN[g][1];
        const double* dzeta = kHexDN[g][2];
        const double xi = (g >> 2) ? kGauss : -kGauss, eta = ((g >> 1) & 1) ? kGauss : -kGauss,
                     zeta = (g & 1) ? kGauss : -kGauss;
        const double xe = (g >> 2) == ((g >> 1) & 1) ? kGauss * kGauss : -(kGauss * kGauss);
        const double xz = (g >> 2) == (g & 1) ? kGauss * kGauss : -(kGauss * kGauss);
        const double ez = ((g >> 1) & 1) == (g & 1) ? kGauss * kGauss : -(kGauss * kGauss);
        double J[3][3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          J[0][q] = fma(ez, mo[q][7], fma(zeta, mo[q][5], fma(eta, mo[q][3], mo[q][1])));
          J[1][q] = fma(xz, mo[q][7], fma(zeta, mo[q][6], fma(xi, mo[q][3], mo[q][2])));
          J[2][q] = fma(xe, mo[q][7], fma(eta, mo[q][6], fma(xi, mo[q][5], mo[q][4])));
        }
        // determinant by the first row, inverse = adjugate / det
        const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        if (bad && !ref::measure_ok(det)) atomicOr(bad, kFlagDegenerateCell);
        const double id = 1.0 / det;
        const double v00 = c00 * id, v10 = c01 * id, v20 = c02 * id;
        const double v01 = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id;
        const double v11 = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id;
        const double v21 = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id;
        const double v02 = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id;
        const double v12 = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id;
        const double v22 = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id;
        // physical gradients, and the same scaled by det for the weighted products
        double dx[8], dy[8], dz[8], sx[8], sy[8], sz[8];
#pragma unroll
        for (int a = 0; a < 8; ++a) {
          dx[a] = v00 * dxi[a] + v01 * deta[a] + v02 * dzeta[a];
          dy[a] = v10 * dxi[a] + v11 * deta[a] + v12 * dzeta[a];
          dz[a] = v20 * dxi[a] + v21 * deta[a] + v22 * dzeta[a];
          sx[a] = dx[a] * det;
          sy[a] = dy[a] * det;
          sz[a] = dz[a] * det;
        }
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int b = a; b < 8; ++b) K[a][b] = fma(sx[a], dx[b], fma(sy[a], dy[b], fma(sz[a], dz[b], K[a][b])));
      }
      if (coeff) {
        const double k = __ldg(coeff + c);
#pragma unroll
        for (int a = 0; a < 8; ++a)
#pragma unroll
          for (int b = a; b < 8; ++b) K[a][b] *= k;
      }
      write_rows_q1<8>(K, inv + 8 * c, er);
    }
  }
}

// Constant source on Quad4 / Hexa8 cells, 2 x 2 (x 2) Gauss points
// (applyConstantSourceToRhsQuad4 / Hexa8, femutils/ArcaneFemFunctionsGpu.cc:
// 393-458,875-960, which adds every Gauss-point term with an atomic).  Each
// (cell, local node, Gauss point) term N_a qdot (w detJ), w = 1, rounded as
// the reference rounds it, goes to its incidence slot term[inv[c][a] * NG + g];
// k_incidence_gp_sum then adds a node's terms in increasing cell order and, per
// cell, in Gauss-point order: the deterministic order of a sequential cell
// loop.  Jacobians in the reference's rounding (afem_elem_ref.cuh).
template <int N>
__global__ void __launch_bounds__(128) k_cell_source_q1(int nb_cell, const double* __restrict__ xyz,
                                                        const int32_t* __restrict__ cn,
                                                        const int32_t* __restrict__ inv, double qdot,
                                                        double* __restrict__ term) {
  constexpr int NG = N;   // 4 Gauss points for Quad4, 8 for Hexa8
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nb_cell; c += (int64_t)gridDim.x * blockDim.x) {
    double x[N], y[N], z[N];
    int32_t pos[N];
#pragma unroll
    for (int a = 0; a < N; ++a) {
      const double* p = xyz + 3 * (int64_t)__ldg(cn + N * c + a);
      x[a] = __ldg(p);
      y[a] = __ldg(p + 1);
      z[a] = __ldg(p + 2);
      pos[a] = __ldg(inv + N * c + a);
    }
#pragma unroll 1
    for (int g = 0; g < NG; ++g) {
      double det;
      const double* Nf;
      if constexpr (N == 4) {
        double J[2][2];
        det = ref::quad4_jacobian(x, y, kQuadDnRef, g, J);
        Nf = kQuadDnRef.N[g];
      } else {
        double J[3][3], mm[3];
        det = ref::hexa8_jacobian(x, y, z, kHexDnRef, g, J, mm);
        Nf = kHexDnRef.N[g];
      }
#pragma unroll
      for (int a = 0; a < N; ++a) term[(int64_t)pos[a] * NG + g] = ref::mul(ref::mul(Nf[a], qdot), det);
    }
  }
}

// rhs[n * nb_dof] = sum of the node's incidence terms, `per` consecutive
// terms per incidence (increasing cell order, then term order)
__global__ void k_incidence_sum(int nb_node, const int32_t* __restrict__ nc_ptr, const double* __restrict__ term,
                                int per, int nb_dof, double* __restrict__ rhs) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nb_node; n += gridDim.x * blockDim.x) {
    double s = 0.0;
    const int64_t t1 = (int64_t)nc_ptr[n + 1] * per;
    for (int64_t t = (int64_t)nc_ptr[n] * per; t < t1; ++t) s = __dadd_rn(s, term[t]);
    rhs[(int64_t)n * nb_dof] = s;
  }
}

// Boundary-face terms (Neumann flux, traction), per face g * |f| / nf, in
// the oracle's operation order with no contraction (applyNeumannToRhsTria3 /
// Tetra4, femutils/ArcaneFemFunctionsGpu.cc:679-735,1082-1140; traction
// femutils/ArcaneFemFunctions.h:2188-2220,2854-2885).  term[f][c].
__global__ void k_face_terms(int dim, int nb_face, const double* __restrict__ xyz, const int32_t* __restrict__ fn,
                             const uint8_t* __restrict__ outward, int mode, double g0, double g1, double g2,
                             double* __restrict__ term) {
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nb_face; f += gridDim.x * blockDim.x) {
    const int32_t* q = fn + (int64_t)f * dim;
    const double* a0 = xyz + 3 * (int64_t)q[0];
    const double* a1 = xyz + 3 * (int64_t)q[1];
    const bool out = outward ? outward[f] != 0 : true;
    const double* b0 = out ? a0 : a1;
    const double* b1 = out ? a1 : a0;
    double measure, n0 = 0.0, n1 = 0.0, n2 = 0.0;
    if (dim == 2) {
      const double dx = __dsub_rn(a1[0], a0[0]), dy = __dsub_rn(a1[1], a0[1]);
      measure = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
      const double ex = __dsub_rn(b1[0], b0[0]), ey = __dsub_rn(b1[1], b0[1]);
      const double nn = __dsqrt_rn(__dadd_rn(__dmul_rn(ey, ey), __dmul_rn(ex, ex)));
      n0 = __ddiv_rn(ey, nn);
      n1 = __ddiv_rn(__dsub_rn(b0[0], b1[0]), nn);
    } else {
      const double* a2 = xyz + 3 * (int64_t)q[2];
      const double u0 = __dsub_rn(a1[0], a0[0]), u1 = __dsub_rn(a1[1], a0[1]), u2 = __dsub_rn(a1[2], a0[2]);
      const double v0 = __dsub_rn(a2[0], a0[0]), v1 = __dsub_rn(a2[1], a0[1]), v2 = __dsub_rn(a2[2], a0[2]);
      const double c0 = __dsub_rn(__dmul_rn(u1, v2), __dmul_rn(u2, v1));
      const double c1 = __dsub_rn(__dmul_rn(u2, v0), __dmul_rn(u0, v2));
      const double c2 = __dsub_rn(__dmul_rn(u0, v1), __dmul_rn(u1, v0));
      measure = __ddiv_rn(__dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(c0, c0), __dmul_rn(c1, c1)), __dmul_rn(c2, c2))),
                          2.0);
      const double e10 = __dsub_rn(b1[0], b0[0]), e11 = __dsub_rn(b1[1], b0[1]), e12 = __dsub_rn(b1[2], b0[2]);
      const double e20 = __dsub_rn(a2[0], b0[0]), e21 = __dsub_rn(a2[1], b0[1]), e22 = __dsub_rn(a2[2], b0[2]);
      const double m0 = __dsub_rn(__dmul_rn(e11, e22), __dmul_rn(e12, e21));
      const double m1 = __dsub_rn(__dmul_rn(e12, e20), __dmul_rn(e10, e22));
      const double m2 = __dsub_rn(__dmul_rn(e10, e21), __dmul_rn(e11, e20));
      const double nn = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(m0, m0), __dmul_rn(m1, m1)), __dmul_rn(m2, m2)));
      n0 = __ddiv_rn(m0, nn);
      n1 = __ddiv_rn(m1, nn);
      n2 = __ddiv_rn(m2, nn);
    }
    const double nf = (double)dim;
    double* t = term + 3 * (int64_t)f;
    if (mode == AFEM_FACE_SCALAR) {
      t[0] = __ddiv_rn(__dmul_rn(g0, measure), nf);
    } else if (mode == AFEM_FACE_NORMAL) {
      double flux = __dadd_rn(__dmul_rn(n0, g0), __dmul_rn(n1, g1));
      if (dim == 3) flux = __dadd_rn(flux, __dmul_rn(n2, g2));
      t[0] = __ddiv_rn(__dmul_rn(flux, measure), nf);
    } else {
      t[0] = __ddiv_rn(__dmul_rn(g0, measure), nf);
      t[1] = __ddiv_rn(__dmul_rn(g1, measure), nf);
      if (dim == 3) t[2] = __ddiv_rn(__dmul_rn(g2, measure), nf);
    }
  }
}

// rhs[n][c] += term of every incident face, in increasing face order.
__global__ void k_face_gather(int nb_node, const int32_t* __restrict__ ptr, const int32_t* __restrict__ face,
                              const double* __restrict__ term, int ncomp, int nb_dof, double* __restrict__ rhs) {
  for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nb_node; n += gridDim.x * blockDim.x) {
    const int32_t p0 = ptr[n], p1 = ptr[n + 1];
    if (p0 == p1) continue;
    for (int c = 0; c < ncomp; ++c) {
      double acc = rhs[(int64_t)n * nb_dof + c];
      for (int32_t p = p0; p < p1; ++p) acc = __dadd_rn(acc, term[3 * (int64_t)face[p] + c]);
      rhs[(int64_t)n * nb_dof + c] = acc;
    }
  }
}

// Cell measure in the reference's rounding: computeAreaTria3 /
// computeVolumeTetra4 (femutils/ArcaneFemFunctionsGpu.h:76-86,113-128).
__device__ __forceinline__ double cell_measure_ref(int dim, const double* __restrict__ xyz,
                                                   const int32_t* __restrict__ cn, int64_t c) {
  const int npc = dim + 1;
  double n[4][3];
  for (int a = 0; a < npc; ++a) {
    const double* p = xyz + 3 * (int64_t)__ldg(cn + npc * c + a);
    n[a][0] = __ldg(p);
    n[a][1] = __ldg(p + 1);
    n[a][2] = __ldg(p + 2);
  }
  if (dim == 2) {
    const double t[3][3] = {{n[0][0], n[0][1], n[0][2]}, {n[1][0], n[1][1], n[1][2]}, {n[2][0], n[2][1], n[2][2]}};
    return ref::tri_area(t);
  }
  return ref::tet_volume(n);
}

// w_c = (qdot * measure) / npc, each operation rounded as the reference's
// sum += qdot * domain / nbItem rounds it (the division by 4 an exact
// scaling, by 3 the corrected constant-reciprocal product).
__global__ void k_cell_source_weight(int nb_cell, int dim, const double* __restrict__ xyz,
                                     const int32_t* __restrict__ cn, double qdot, double* __restrict__ w) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nb_cell; c += (int64_t)gridDim.x * blockDim.x) {
    const double qm = __dmul_rn(qdot, cell_measure_ref(dim, xyz, cn, c));
    w[c] = dim == 3 ? ref::div_const<4>(qm) : ref::div_const<3>(qm);
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
      const double wc = w[nc_cell[p]];
      sum = __dadd_rn(sum, body ? __dmul_rn(__dmul_rn(f, wc), 0.25) : wc);   // f * volume / 4 (exact quarter)
    }
    rhs[d] = sum;
  }
}

__global__ void k_cell_volume(int nb_cell, const double* __restrict__ xyz, const int32_t* __restrict__ cn,
                              double* __restrict__ vol) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < nb_cell; c += (int64_t)gridDim.x * blockDim.x)
    vol[c] = cell_measure_ref(3, xyz, cn, c);
}

static afem_status check_mesh(const afem_mesh_view* m, const char* who) {
  AFEM_CHECK_ARG(m != nullptr, "%s: null mesh view", who);
  AFEM_CHECK_ARG(m->dim == 2 || m->dim == 3, "%s: dim must be 2 or 3 (got %d)", who, m->dim);
  AFEM_CHECK_ARG(m->nb_node > 0 && m->nb_cell > 0, "%s: empty mesh", who);
  AFEM_CHECK_ARG(m->coords_d && m->cell_nodes_d && m->nc_ptr_d && m->nc_cell_d, "%s: null mesh buffer", who);
  if (m->dim == 3)
    AFEM_CHECK_ARG(((uintptr_t)m->cell_nodes_d & 15) == 0, "%s: cell_nodes must be 16-byte aligned", who);
  return AFEM_OK;
}

static afem_status check_assembly(const afem_mesh_view* m, const char* who) {
  AFEM_TRY(check_mesh(m, who));
  AFEM_CHECK_ARG(m->nc_inverse_d && m->nc_slot_d, "%s: null nc_inverse / nc_slot", who);
  if (m->dim == 3)
    AFEM_CHECK_ARG(((uintptr_t)m->nc_inverse_d & 15) == 0 && ((uintptr_t)m->nc_slot_d & 3) == 0,
                   "%s: nc_inverse must be 16-byte and nc_slot 4-byte aligned", who);
  return AFEM_OK;
}

}  // namespace afem

namespace afem {
// L1 for the scalar gathers.  Each thread streams its own row's element rows
// (32 B per incidence), so a warp's loads touch 32 separate lines that are
// re-read over the next incidences; with the default carveout nearly all of
// the SM's 256 KB go to the shared-memory accumulators (7 blocks x 32 KB) and
// the lines are evicted before their reuse.  A 50 % shared-memory carveout
// keeps 4 blocks (16 warps) resident and leaves ~120 KB of L1.  Measured at
// 128^3 / 96^3 (gather ms, carveout 25 / 40 / 50 / 60 / 75 / 100 %):
// tetrahedra 1.28 / 0.59 / 0.56 / 0.57 / 0.62 / 1.02 (default 1.00), Hexa8
// 0.50 / 0.38 / 0.37 / 0.36 / 0.37 / 0.50 (default 0.50).  The elasticity
// gather is best at its default (1.90 ms; 1.92 at 75 %, 2.48 at 50 %).
// The attribute belongs to the device that is current when it is set, so it
// is set once per device (bit d of g_gather_attrs_set), on first use there.
static std::atomic<uint64_t> g_gather_attrs_set{0};
static void gather_attrs() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  const uint64_t bit = uint64_t(1) << dev;
  if (g_gather_attrs_set.load(std::memory_order_acquire) & bit) return;
  cudaFuncSetAttribute(k_gather_scalar<3>, cudaFuncAttributePreferredSharedMemoryCarveout, 50);
  cudaFuncSetAttribute(k_gather_scalar<4>, cudaFuncAttributePreferredSharedMemoryCarveout, 50);
  cudaFuncSetAttribute(k_gather_scalar<8>, cudaFuncAttributePreferredSharedMemoryCarveout, 50);
  g_gather_attrs_set.fetch_or(bit, std::memory_order_acq_rel);
}
}  // namespace afem

namespace afem {
// Element-kernel launches over cells [c0, c1), by the context's formulation.
// The reference-rounding kernels hold more live values (about 130 registers
// per thread), so they run 128-thread blocks.
static afem_status launch_elem_p1(afem_context ctx, const afem_mesh_view* m, int c0, int c1, const double* coeff,
                                  double* ke) {
  const int f = ctx->formulation;
  int* bad = ctx->flags_d;
  if (f == AFEM_FORMULATION_MINIMAL) {
    const unsigned ge = grid_for(ctx, c1 - c0, 256, 16);
    if (m->dim == 3)
      return launch(ctx, k_elem_poisson_tet, ge, 256, 0, c0, c1, m->coords_d, m->cell_nodes_d, m->nc_inverse_d, coeff,
                    ke, bad);
    return launch(ctx, k_elem_poisson_tri, ge, 256, 0, c0, c1, m->coords_d, m->cell_nodes_d, m->nc_inverse_d, coeff, ke,
                  bad);
  }
  const unsigned ge = grid_for(ctx, c1 - c0, 128, 32);
  if (m->dim == 3)
    return f == AFEM_FORMULATION_TESTLAB
               ? launch(ctx, k_elem_poisson_p1_ref<4, AFEM_FORMULATION_TESTLAB>, ge, 128, 0, c0, c1, m->coords_d,
                        m->cell_nodes_d, m->nc_inverse_d, coeff, ke, bad)
               : launch(ctx, k_elem_poisson_p1_ref<4, AFEM_FORMULATION_REFERENCE>, ge, 128, 0, c0, c1, m->coords_d,
                        m->cell_nodes_d, m->nc_inverse_d, coeff, ke, bad);
  return f == AFEM_FORMULATION_TESTLAB
             ? launch(ctx, k_elem_poisson_p1_ref<3, AFEM_FORMULATION_TESTLAB>, ge, 128, 0, c0, c1, m->coords_d,
                      m->cell_nodes_d, m->nc_inverse_d, coeff, ke, bad)
             : launch(ctx, k_elem_poisson_p1_ref<3, AFEM_FORMULATION_REFERENCE>, ge, 128, 0, c0, c1, m->coords_d,
                      m->cell_nodes_d, m->nc_inverse_d, coeff, ke, bad);
}

static afem_status launch_elem_q1(afem_context ctx, const afem_mesh_view* m, int c0, int c1, const double* coeff,
                                  double* ke) {
  const bool minimal = ctx->formulation == AFEM_FORMULATION_MINIMAL;
  int* bad = ctx->flags_d;
  const unsigned ge = grid_for(ctx, c1 - c0, 128, 16);
  if (m->dim == 3)
    return minimal ? launch(ctx, k_elem_poisson_hexa8<AFEM_FORMULATION_MINIMAL>, ge, 128, 0, c0, c1, m->coords_d,
                            m->cell_nodes_d, m->nc_inverse_d, coeff, ke, bad)
                   : launch(ctx, k_elem_poisson_hexa8<AFEM_FORMULATION_REFERENCE>, ge, 128, 0, c0, c1, m->coords_d,
                            m->cell_nodes_d, m->nc_inverse_d, coeff, ke, bad);
  return minimal ? launch(ctx, k_elem_poisson_quad4<AFEM_FORMULATION_MINIMAL>, ge, 128, 0, c0, c1, m->coords_d,
                          m->cell_nodes_d, m->nc_inverse_d, coeff, ke, bad)
                 : launch(ctx, k_elem_poisson_quad4<AFEM_FORMULATION_REFERENCE>, ge, 128, 0, c0, c1, m->coords_d,
                          m->cell_nodes_d, m->nc_inverse_d, coeff, ke, bad);
}

static afem_status launch_elem_elasticity(afem_context ctx, const afem_mesh_view* m, int c0, int c1, double lambda,
                                          double mu, double* ke) {
  const unsigned ge = grid_for(ctx, c1 - c0, kElastElemBlock, 32);
  if (ctx->formulation == AFEM_FORMULATION_MINIMAL)
    return launch(ctx, k_elem_elasticity_tet<AFEM_FORMULATION_MINIMAL>, ge, kElastElemBlock, 0, c0, c1, m->coords_d,
                  m->cell_nodes_d, m->nc_inverse_d, lambda, mu, ke, ctx->flags_d);
  return launch(ctx, k_elem_elasticity_tet<AFEM_FORMULATION_REFERENCE>, ge, kElastElemBlock, 0, c0, c1, m->coords_d,
                m->cell_nodes_d, m->nc_inverse_d, lambda, mu, ke, ctx->flags_d);
}
}  // namespace afem

using namespace afem;

extern "C" {

afem_status afem_element_matrices_poisson_p1(afem_context ctx, const afem_mesh_view* m, const double* cell_coeff_d,
                                             double* ke) {
  AFEM_CHECK_ARG(ctx, "afem_element_matrices_poisson_p1: null context");
  AFEM_TRY(check_assembly(m, "afem_element_matrices_poisson_p1"));
  AFEM_CHECK_ARG(ke && ((uintptr_t)ke & 31) == 0, "afem_element_matrices_poisson_p1: ke null or not 32-byte aligned");
  return launch_elem_p1(ctx, m, 0, m->nb_cell, cell_coeff_d, ke);
}

afem_status afem_gather_poisson_p1(afem_context ctx, const afem_mesh_view* m, const int32_t* row_ptr_d,
                                   const double* ke, double* values_d) {
  gather_attrs();
  AFEM_CHECK_ARG(ctx, "afem_gather_poisson_p1: null context");
  AFEM_TRY(check_assembly(m, "afem_gather_poisson_p1"));
  AFEM_CHECK_ARG(row_ptr_d && ke && values_d && ((uintptr_t)ke & 31) == 0, "afem_gather_poisson_p1: bad buffer");
  unsigned gg = (unsigned)((m->nb_node + kGatherBlock - 1) / kGatherBlock);
  if (m->dim == 3)
    return launch(ctx, k_gather_scalar<4>, gg, kGatherBlock, 0, 0, m->nb_node, m->nc_ptr_d, m->nc_slot_d, row_ptr_d, ke,
                  values_d);
  return launch(ctx, k_gather_scalar<3>, gg, kGatherBlock, 0, 0, m->nb_node, m->nc_ptr_d, m->nc_slot_d, row_ptr_d, ke,
                values_d);
}


// Range count for chunks == 0: one range per ~80 MB of values, at most 12.
// Measured on GB300 at ~193 GB/s device -> host: fewer ranges leave a longer
// copy of the last range after the compute; more ranges add per-range launch
// and synchronisation cost (3D Poisson, 254 MB: best at 4; elasticity,
// 970 MB: best at 12, slower at 16).
constexpr double kAutoRangeBytes = 80e6;
constexpr double kRangeRatio = 0.6;   // successive cell-range sizes of the scalar pipelined assembly
constexpr int kAutoMaxRanges = 12;

static afem_status auto_ranges(afem_context ctx, const int32_t* row_ptr_d, int n, int64_t scale, int* chunks) {
  int32_t* hb = reinterpret_cast<int32_t*>(ctx->pinned);
  AFEM_CUDA(cudaMemcpyAsync(hb, row_ptr_d + n, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
  const double bytes = (double)hb[0] * (double)scale * sizeof(double);
  *chunks = (int)std::min<double>(kAutoMaxRanges, std::max(1.0, std::ceil(bytes / kAutoRangeBytes)));
  return AFEM_OK;
}

afem_status afem_gather_to_host(afem_context ctx, const afem_mesh_view* m, int kind, const int32_t* row_ptr_d,
                                const double* ke, int layout, double* values_d, double* values_h, int chunks) {
  gather_attrs();
  AFEM_CHECK_ARG(ctx, "afem_gather_to_host: null context");
  AFEM_TRY(check_assembly(m, "afem_gather_to_host"));
  AFEM_CHECK_ARG(row_ptr_d && ke && values_d && values_h && ((uintptr_t)ke & 31) == 0,
                 "afem_gather_to_host: bad buffer");
  AFEM_CHECK_ARG(chunks >= 0 && chunks <= 16, "afem_gather_to_host: chunks 0..16");
  AFEM_CHECK_ARG(kind == AFEM_GATHER_POISSON_P1 || kind == AFEM_GATHER_POISSON_Q1 ||
                     (kind == AFEM_GATHER_ELASTICITY_TET4 && m->dim == 3),
                 "afem_gather_to_host: bad kind %d", kind);
  AFEM_CHECK_ARG(kind != AFEM_GATHER_ELASTICITY_TET4 || layout == AFEM_LAYOUT_PER_BLOCK ||
                     layout == AFEM_LAYOUT_PER_ROW,
                 "afem_gather_to_host: bad layout %d", layout);
  if (chunks == 0)
    AFEM_TRY(auto_ranges(ctx, row_ptr_d, m->nb_node, kind == AFEM_GATHER_ELASTICITY_TET4 ? 9 : 1, &chunks));
  if (!ctx->copy_stream) AFEM_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  for (int k = 0; k <= chunks; ++k)
    if (!ctx->chunk_ev[k]) AFEM_CUDA(cudaEventCreateWithFlags(&ctx->chunk_ev[k], cudaEventDisableTiming));
  cudaStream_t s = ctx->stream, cs = ctx->copy_stream;
  // chunk boundaries (nodes) and their value offsets; the copy stream waits for
  // everything queued so far on the context stream (row_ptr may be fresh)
  const int n = m->nb_node;
  const int per = (n + chunks - 1) / chunks;
  int32_t* hb = reinterpret_cast<int32_t*>(ctx->pinned);   // 256 bytes: up to 64 entries
  AFEM_CUDA(cudaEventRecord(ctx->chunk_ev[0], s));
  AFEM_CUDA(cudaStreamWaitEvent(cs, ctx->chunk_ev[0], 0));
  for (int k = 0; k <= chunks; ++k)
    AFEM_CUDA(cudaMemcpyAsync(hb + k, row_ptr_d + std::min(k * per, n), sizeof(int32_t), cudaMemcpyDeviceToHost, cs));
  AFEM_CUDA(cudaStreamSynchronize(cs));
  int64_t off[17];
  for (int k = 0; k <= chunks; ++k) off[k] = hb[k];
  const int64_t scale = kind == AFEM_GATHER_ELASTICITY_TET4 ? 9 : 1;   // values per block entry
  const int npc = kind == AFEM_GATHER_POISSON_Q1 ? (1 << m->dim) : m->dim + 1;
  for (int k = 0; k < chunks; ++k) {
    const int n0 = std::min(k * per, n), n1 = std::min((k + 1) * per, n);
    if (n1 <= n0) continue;
    if (kind == AFEM_GATHER_ELASTICITY_TET4) {
      const unsigned gg = (unsigned)((3 * (int64_t)(n1 - n0) + kGatherBlock - 1) / kGatherBlock);
      AFEM_TRY(launch(ctx, k_gather_elasticity, gg, kGatherBlock, 0, n0, n1, m->nc_ptr_d, m->nc_slot_d, row_ptr_d,
                      ke, (int)(layout == AFEM_LAYOUT_PER_ROW), values_d));
    } else {
      const unsigned gg = (unsigned)((n1 - n0 + kGatherBlock - 1) / kGatherBlock);
      auto kern = npc == 8 ? k_gather_scalar<8> : npc == 4 ? k_gather_scalar<4> : k_gather_scalar<3>;
      AFEM_TRY(launch(ctx, kern, gg, kGatherBlock, 0, n0, n1, m->nc_ptr_d, m->nc_slot_d, row_ptr_d, ke, values_d));
    }
    AFEM_CUDA(cudaEventRecord(ctx->chunk_ev[k + 1], s));
    AFEM_CUDA(cudaStreamWaitEvent(cs, ctx->chunk_ev[k + 1], 0));
    const int64_t v0 = off[k] * scale, v1 = off[k + 1] * scale;
    if (v1 > v0)
      AFEM_CUDA(cudaMemcpyAsync(values_h + v0, values_d + v0, sizeof(double) * (size_t)(v1 - v0),
                                cudaMemcpyDeviceToHost, cs));
  }
  AFEM_CUDA(cudaStreamSynchronize(cs));
  return check_flags(ctx);
}

}  // extern "C"

// afem_assemble_to_host, and with coords_h (afem_assemble_host_io) the node
// coordinates uploaded into mesh->coords_d in node prefixes on a third stream:
// the cells below a range's end use only nodes up to the last one whose first
// incident cell lies below it (k_node_bounds' `need`), so each prefix is
// copied ahead of the first cell range that needs it while earlier ranges
// compute.
static afem_status assemble_to_host_impl(afem_context ctx, const afem_mesh_view* m, int kind,
                                         const int32_t* row_ptr_d, const double* cell_coeff_d, double lambda,
                                         double mu, int layout, double* ke, double* values_d, double* values_h,
                                         int chunks, const double* coords_h) {
  gather_attrs();
  AFEM_CHECK_ARG(ctx, "afem_assemble_to_host: null context");
  AFEM_TRY(check_assembly(m, "afem_assemble_to_host"));
  AFEM_CHECK_ARG(row_ptr_d && ke && values_d && values_h && ((uintptr_t)ke & 31) == 0,
                 "afem_assemble_to_host: bad buffer");
  AFEM_CHECK_ARG(chunks >= 0 && chunks <= kMaxAsmChunks, "afem_assemble_to_host: chunks 0..%d", kMaxAsmChunks);
  AFEM_CHECK_ARG(kind == AFEM_GATHER_POISSON_P1 || kind == AFEM_GATHER_POISSON_Q1 ||
                     (kind == AFEM_GATHER_ELASTICITY_TET4 && m->dim == 3),
                 "afem_assemble_to_host: bad kind %d", kind);
  AFEM_CHECK_ARG(kind != AFEM_GATHER_ELASTICITY_TET4 || layout == AFEM_LAYOUT_PER_BLOCK ||
                     layout == AFEM_LAYOUT_PER_ROW,
                 "afem_assemble_to_host: bad layout %d", layout);
  AFEM_CHECK_ARG(m->nc_ptr_d && m->nc_cell_d, "afem_assemble_to_host: null node->cell lists");
  if (chunks == 0)
    AFEM_TRY(auto_ranges(ctx, row_ptr_d, m->nb_node, kind == AFEM_GATHER_ELASTICITY_TET4 ? 9 : 1, &chunks));
  if (!ctx->copy_stream) AFEM_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
  for (int k = 0; k <= chunks; ++k)
    if (!ctx->chunk_ev[k]) AFEM_CUDA(cudaEventCreateWithFlags(&ctx->chunk_ev[k], cudaEventDisableTiming));
  cudaStream_t s = ctx->stream, cs = ctx->copy_stream;
  const int nc = m->nb_cell, nn = m->nb_node;
  // cell chunks and the node prefixes they complete
  CellBounds cb{};
  int64_t cbound[kMaxAsmChunks + 1];
  // Scalar kinds produce values more slowly than the link copies them back, so only the last range's copy is
  // exposed: range sizes shrink geometrically (ratio kRangeRatio) to keep it short.  Elasticity's copy is longer
  // than its compute: equal ranges start the copies earliest.
  if (kind == AFEM_GATHER_ELASTICITY_TET4) {
    for (int k = 0; k <= chunks; ++k) cbound[k] = (int64_t)nc * k / chunks;
  } else {
    double w[kMaxAsmChunks + 1], tot = 0.0, acc = 0.0;
    for (int k = 0; k < chunks; ++k) tot += (w[k] = std::pow(kRangeRatio, k));
    cbound[0] = 0;
    for (int k = 0; k < chunks; ++k) {
      acc += w[k];
      cbound[k + 1] = k + 1 == chunks ? nc : std::min<int64_t>(nc, (int64_t)(nc * (acc / tot)));
    }
  }
  for (int k = 1; k < chunks; ++k) cb.b[k - 1] = (int32_t)cbound[k];
  AFEM_TRY(scratch_reserve(ctx, 512));
  int32_t *first, *need;
  AFEM_TRY(scratch_take(ctx, kMaxAsmChunks + 1, &first));
  AFEM_TRY(scratch_take(ctx, kMaxAsmChunks + 1, &need));
  // 64 pinned ints: node bounds at 0, coordinate needs at 16, row starts at 32
  int32_t* hb = reinterpret_cast<int32_t*>(ctx->pinned);
  int32_t nb[kMaxAsmChunks + 1], upto[kMaxAsmChunks + 1];
  nb[0] = 0;
  nb[chunks] = nn;
  upto[chunks - 1] = nn;   // the last range: every node
  if (chunks > 1) {
    AFEM_CUDA(cudaMemsetAsync(first, 0x7f, sizeof(int32_t) * (chunks - 1), s));
    if (coords_h) AFEM_CUDA(cudaMemsetAsync(need, 0xff, sizeof(int32_t) * (chunks - 1), s));
    AFEM_TRY(launch(ctx, k_node_bounds, grid_for(ctx, nn, 256), 256, 0, nn, m->nc_ptr_d, m->nc_cell_d, chunks - 1, cb,
                    first, coords_h ? need : (int32_t*)nullptr));
    AFEM_CUDA(cudaMemcpyAsync(hb, first, sizeof(int32_t) * (chunks - 1), cudaMemcpyDeviceToHost, s));
    if (coords_h)
      AFEM_CUDA(cudaMemcpyAsync(hb + 16, need, sizeof(int32_t) * (chunks - 1), cudaMemcpyDeviceToHost, s));
    AFEM_CUDA(cudaStreamSynchronize(s));
    for (int k = 1; k < chunks; ++k) nb[k] = std::min(std::max(hb[k - 1], nb[k - 1]), nn);   // monotone
    if (coords_h)
      for (int k = 0; k + 1 < chunks; ++k) upto[k] = std::min(std::max(hb[16 + k] + 1, k ? upto[k - 1] : 0), nn);
  }
  // coordinate uploads, each ahead of the first range that needs it (h2d_at[k]: the event range k waits for)
  int h2d_at[kMaxAsmChunks];
  if (coords_h) {
    if (!ctx->h2d_stream) AFEM_CUDA(cudaStreamCreateWithFlags(&ctx->h2d_stream, cudaStreamNonBlocking));
    for (int k = 0; k <= chunks; ++k)
      if (!ctx->h2d_ev[k]) AFEM_CUDA(cudaEventCreateWithFlags(&ctx->h2d_ev[k], cudaEventDisableTiming));
    // earlier work of the context stream may still read the coordinates
    AFEM_CUDA(cudaEventRecord(ctx->h2d_ev[chunks], s));
    AFEM_CUDA(cudaStreamWaitEvent(ctx->h2d_stream, ctx->h2d_ev[chunks], 0));
    double* coords_d = const_cast<double*>(m->coords_d);
    int uploaded = 0, last = -1;
    for (int k = 0; k < chunks; ++k) {
      if (upto[k] > uploaded) {
        AFEM_CUDA(cudaMemcpyAsync(coords_d + 3 * (int64_t)uploaded, coords_h + 3 * (int64_t)uploaded,
                                  sizeof(double) * 3 * (size_t)(upto[k] - uploaded), cudaMemcpyHostToDevice,
                                  ctx->h2d_stream));
        AFEM_CUDA(cudaEventRecord(ctx->h2d_ev[k], ctx->h2d_stream));
        uploaded = upto[k];
        last = k;
      }
      h2d_at[k] = last;
    }
  }
  for (int k = 0; k <= chunks; ++k)
    AFEM_CUDA(cudaMemcpyAsync(hb + 32 + k, row_ptr_d + nb[k], sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  AFEM_CUDA(cudaStreamSynchronize(s));
  int64_t off[kMaxAsmChunks + 1];
  const int64_t scale = kind == AFEM_GATHER_ELASTICITY_TET4 ? 9 : 1;
  for (int k = 0; k <= chunks; ++k) off[k] = (int64_t)hb[32 + k] * scale;
  const int per_row = kind == AFEM_GATHER_ELASTICITY_TET4 ? 3 : 1;
  for (int k = 0; k < chunks; ++k) {
    const int c0 = (int)cbound[k], c1 = (int)cbound[k + 1];
    if (coords_h && h2d_at[k] >= 0 && (k == 0 || h2d_at[k] != h2d_at[k - 1]))
      AFEM_CUDA(cudaStreamWaitEvent(s, ctx->h2d_ev[h2d_at[k]], 0));
    if (c1 > c0) {
      if (kind == AFEM_GATHER_ELASTICITY_TET4)
        AFEM_TRY(launch_elem_elasticity(ctx, m, c0, c1, lambda, mu, ke));
      else if (kind == AFEM_GATHER_POISSON_Q1)
        AFEM_TRY(launch_elem_q1(ctx, m, c0, c1, cell_coeff_d, ke));
      else
        AFEM_TRY(launch_elem_p1(ctx, m, c0, c1, cell_coeff_d, ke));
    }
    const int n0 = nb[k], n1 = nb[k + 1];
    if (n1 > n0) {
      const unsigned gg = (unsigned)(((int64_t)(n1 - n0) * per_row + kGatherBlock - 1) / kGatherBlock);
      if (kind == AFEM_GATHER_ELASTICITY_TET4)
        AFEM_TRY(launch(ctx, k_gather_elasticity, gg, kGatherBlock, 0, n0, n1, m->nc_ptr_d, m->nc_slot_d, row_ptr_d, ke,
                        (int)(layout == AFEM_LAYOUT_PER_ROW), values_d));
      else {
        // incidences per cell: 3 / 4 (P1 triangle / tetrahedron), 4 / 8 (Quad4 / Hexa8)
        const int npc = kind == AFEM_GATHER_POISSON_Q1 ? (1 << m->dim) : m->dim + 1;
        auto kern = npc == 8 ? k_gather_scalar<8> : npc == 4 ? k_gather_scalar<4> : k_gather_scalar<3>;
        AFEM_TRY(launch(ctx, kern, gg, kGatherBlock, 0, n0, n1, m->nc_ptr_d, m->nc_slot_d, row_ptr_d, ke, values_d));
      }
      AFEM_CUDA(cudaEventRecord(ctx->chunk_ev[k + 1], s));
      AFEM_CUDA(cudaStreamWaitEvent(cs, ctx->chunk_ev[k + 1], 0));
      if (off[k + 1] > off[k])
        AFEM_CUDA(cudaMemcpyAsync(values_h + off[k], values_d + off[k], sizeof(double) * (size_t)(off[k + 1] - off[k]),
                                  cudaMemcpyDeviceToHost, cs));
    }
  }
  AFEM_CUDA(cudaStreamSynchronize(cs));
  AFEM_CUDA(cudaStreamSynchronize(s));
  return check_flags(ctx);
}

extern "C" {

afem_status afem_assemble_to_host(afem_context ctx, const afem_mesh_view* m, int kind, const int32_t* row_ptr_d,
                                  const double* cell_coeff_d, double lambda, double mu, int layout, double* ke,
                                  double* values_d, double* values_h, int chunks) {
  return assemble_to_host_impl(ctx, m, kind, row_ptr_d, cell_coeff_d, lambda, mu, layout, ke, values_d, values_h,
                               chunks, nullptr);
}

afem_status afem_assemble_host_io(afem_context ctx, const afem_mesh_view* m, const double* coords_h, int kind,
                                  const int32_t* row_ptr_d, const double* cell_coeff_d, double lambda, double mu,
                                  int layout, double* ke, double* values_d, double* values_h, int chunks) {
  AFEM_CHECK_ARG(coords_h, "afem_assemble_host_io: null host coordinates");
  return assemble_to_host_impl(ctx, m, kind, row_ptr_d, cell_coeff_d, lambda, mu, layout, ke, values_d, values_h,
                               chunks, coords_h);
}

afem_status afem_element_matrices_poisson_q1(afem_context ctx, const afem_mesh_view* m, const double* cell_coeff_d,
                                             double* ke) {
  AFEM_CHECK_ARG(ctx, "afem_element_matrices_poisson_q1: null context");
  AFEM_TRY(check_mesh(m, "afem_element_matrices_poisson_q1"));
  AFEM_CHECK_ARG(m->nc_inverse_d && ke, "afem_element_matrices_poisson_q1: null nc_inverse / element buffer");
  return launch_elem_q1(ctx, m, 0, m->nb_cell, cell_coeff_d, ke);
}

afem_status afem_gather_poisson_q1(afem_context ctx, const afem_mesh_view* m, const int32_t* row_ptr_d,
                                   const double* ke, double* values_d) {
  gather_attrs();
  AFEM_CHECK_ARG(ctx, "afem_gather_poisson_q1: null context");
  AFEM_TRY(check_mesh(m, "afem_gather_poisson_q1"));
  AFEM_CHECK_ARG(m->nc_slot_d && row_ptr_d && ke && values_d, "afem_gather_poisson_q1: null buffer");
  unsigned gg = (unsigned)((m->nb_node + kGatherBlock - 1) / kGatherBlock);
  if (m->dim == 3)
    return launch(ctx, k_gather_scalar<8>, gg, kGatherBlock, 0, 0, m->nb_node, m->nc_ptr_d, m->nc_slot_d, row_ptr_d, ke,
                  values_d);
  return launch(ctx, k_gather_scalar<4>, gg, kGatherBlock, 0, 0, m->nb_node, m->nc_ptr_d, m->nc_slot_d, row_ptr_d, ke,
                values_d);
}

afem_status afem_assemble_poisson_q1(afem_context ctx, const afem_mesh_view* m, const int32_t* row_ptr_d,
                                     const double* cell_coeff_d, double* values_d) {
  gather_attrs();
  AFEM_CHECK_ARG(ctx, "afem_assemble_poisson_q1: null context");
  AFEM_TRY(check_mesh(m, "afem_assemble_poisson_q1"));
  AFEM_CHECK_ARG(row_ptr_d && values_d, "afem_assemble_poisson_q1: null buffer");
  const size_t npc = (size_t)1 << m->dim;
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(double) * npc * npc * m->nb_cell)));
  double* ke;
  AFEM_TRY(scratch_take(ctx, npc * npc * m->nb_cell, &ke));
  AFEM_TRY(afem_element_matrices_poisson_q1(ctx, m, cell_coeff_d, ke));
  return afem_gather_poisson_q1(ctx, m, row_ptr_d, ke, values_d);
}

afem_status afem_assemble_poisson_p1(afem_context ctx, const afem_mesh_view* m, const int32_t* row_ptr_d,
                                     const double* cell_coeff_d, double* values_d) {
  gather_attrs();
  AFEM_CHECK_ARG(ctx, "afem_assemble_poisson_p1: null context");
  AFEM_TRY(check_assembly(m, "afem_assemble_poisson_p1"));
  AFEM_CHECK_ARG(row_ptr_d && values_d, "afem_assemble_poisson_p1: null buffer");
  const size_t npc = m->dim + 1;
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(double) * npc * npc * m->nb_cell)));
  double* ke;
  AFEM_TRY(scratch_take(ctx, npc * npc * m->nb_cell, &ke));
  AFEM_TRY(afem_element_matrices_poisson_p1(ctx, m, cell_coeff_d, ke));
  return afem_gather_poisson_p1(ctx, m, row_ptr_d, ke, values_d);
}

afem_status afem_element_matrices_elasticity_tet4(afem_context ctx, const afem_mesh_view* m, double lambda,
                                                  double mu, double* ke) {
  AFEM_CHECK_ARG(ctx, "afem_element_matrices_elasticity_tet4: null context");
  AFEM_TRY(check_assembly(m, "afem_element_matrices_elasticity_tet4"));
  AFEM_CHECK_ARG(m->dim == 3, "afem_element_matrices_elasticity_tet4: tetrahedra only (dim 3)");
  AFEM_CHECK_ARG(ke && ((uintptr_t)ke & 31) == 0, "afem_element_matrices_elasticity_tet4: ke null or misaligned");
  return launch_elem_elasticity(ctx, m, 0, m->nb_cell, lambda, mu, ke);
}

afem_status afem_gather_elasticity_tet4(afem_context ctx, const afem_mesh_view* m, const int32_t* row_ptr_d,
                                        const double* ke, int layout, double* values_d) {
  gather_attrs();
  AFEM_CHECK_ARG(ctx, "afem_gather_elasticity_tet4: null context");
  AFEM_TRY(check_assembly(m, "afem_gather_elasticity_tet4"));
  AFEM_CHECK_ARG(m->dim == 3, "afem_gather_elasticity_tet4: tetrahedra only (dim 3)");
  AFEM_CHECK_ARG(layout == AFEM_LAYOUT_PER_BLOCK || layout == AFEM_LAYOUT_PER_ROW,
                 "afem_gather_elasticity_tet4: bad layout %d", layout);
  AFEM_CHECK_ARG(row_ptr_d && ke && values_d && ((uintptr_t)ke & 31) == 0, "afem_gather_elasticity_tet4: bad buffer");
  unsigned gg = (unsigned)((3 * (int64_t)m->nb_node + kGatherBlock - 1) / kGatherBlock);
  return launch(ctx, k_gather_elasticity, gg, kGatherBlock, 0, 0, m->nb_node, m->nc_ptr_d, m->nc_slot_d, row_ptr_d, ke,
                (int)(layout == AFEM_LAYOUT_PER_ROW), values_d);
}

afem_status afem_assemble_elasticity_tet4(afem_context ctx, const afem_mesh_view* m, const int32_t* row_ptr_d,
                                          double lambda, double mu, int layout, double* values_d) {
  AFEM_CHECK_ARG(ctx, "afem_assemble_elasticity_tet4: null context");
  AFEM_TRY(check_assembly(m, "afem_assemble_elasticity_tet4"));
  AFEM_CHECK_ARG(row_ptr_d && values_d, "afem_assemble_elasticity_tet4: null buffer");
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(double) * (size_t)144 * m->nb_cell)));
  double* ke;
  AFEM_TRY(scratch_take(ctx, (size_t)144 * m->nb_cell, &ke));
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

afem_status afem_rhs_constant_source_q1(afem_context ctx, const afem_mesh_view* m, double qdot, int nb_dof,
                                        double* rhs_d) {
  AFEM_CHECK_ARG(ctx, "afem_rhs_constant_source_q1: null context");
  AFEM_TRY(check_mesh(m, "afem_rhs_constant_source_q1"));
  AFEM_CHECK_ARG(m->nc_inverse_d && nb_dof >= 1 && rhs_d, "afem_rhs_constant_source_q1: bad arguments");
  const size_t npc = (size_t)1 << m->dim;   // also the Gauss points per cell
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(double) * npc * npc * (size_t)m->nb_cell)));
  double* term;
  AFEM_TRY(scratch_take(ctx, npc * npc * (size_t)m->nb_cell, &term));
  if (m->dim == 3)
    AFEM_TRY(launch(ctx, k_cell_source_q1<8>, grid_for(ctx, m->nb_cell, 128, 16), 128, 0, m->nb_cell, m->coords_d,
                    m->cell_nodes_d, m->nc_inverse_d, qdot, term));
  else
    AFEM_TRY(launch(ctx, k_cell_source_q1<4>, grid_for(ctx, m->nb_cell, 128, 16), 128, 0, m->nb_cell, m->coords_d,
                    m->cell_nodes_d, m->nc_inverse_d, qdot, term));
  return launch(ctx, k_incidence_sum, grid_for(ctx, m->nb_node, 256), 256, 0, m->nb_node, m->nc_ptr_d,
                (const double*)term, (int)npc, nb_dof, rhs_d);
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

afem_status afem_rhs_boundary_faces(afem_context ctx, int dim, int nb_node, int nb_face, const double* coords_d,
                                    const int32_t* face_nodes_d, const uint8_t* outward_d, int mode,
                                    const double* g_h, int nb_dof, double* rhs_d) {
  AFEM_CHECK_ARG(ctx, "afem_rhs_boundary_faces: null context");
  AFEM_CHECK_ARG(dim == 2 || dim == 3, "afem_rhs_boundary_faces: dim must be 2 or 3");
  AFEM_CHECK_ARG(mode >= AFEM_FACE_SCALAR && mode <= AFEM_FACE_VECTOR, "afem_rhs_boundary_faces: bad mode %d", mode);
  AFEM_CHECK_ARG(nb_node > 0 && nb_face >= 0 && g_h && rhs_d, "afem_rhs_boundary_faces: bad arguments");
  AFEM_CHECK_ARG(nb_dof >= (mode == AFEM_FACE_VECTOR ? dim : 1), "afem_rhs_boundary_faces: nb_dof too small");
  if (nb_face == 0) return AFEM_OK;
  AFEM_CHECK_ARG(coords_d && face_nodes_d, "afem_rhs_boundary_faces: null mesh arrays");
  cudaStream_t s = ctx->stream;
  const size_t total = (size_t)nb_face * dim;
  int32_t *ptr = nullptr, *face = nullptr, *inv = nullptr;
  uint8_t* local = nullptr;
  double* term = nullptr;
  auto release = [&]() {
    if (ptr) cudaFreeAsync(ptr, s);
    if (face) cudaFreeAsync(face, s);
    if (inv) cudaFreeAsync(inv, s);
    if (local) cudaFreeAsync(local, s);
    if (term) cudaFreeAsync(term, s);
  };
  cudaError_t e = cudaMallocAsync((void**)&ptr, sizeof(int32_t) * (nb_node + 1), s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&face, sizeof(int32_t) * total, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&inv, sizeof(int32_t) * total, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&local, total, s);
  if (e == cudaSuccess) e = cudaMallocAsync((void**)&term, sizeof(double) * 3 * nb_face, s);
  if (e != cudaSuccess) {
    release();
    return cuda_fail(e, "afem_rhs_boundary_faces allocation", __FILE__, __LINE__);
  }
  // node -> face incidence in increasing face order (the faces' sequential order)
  afem_status st = afem_node_cell_build(ctx, nb_node, nb_face, dim, face_nodes_d, ptr, face, local, inv);
  // the scalar mode reads g_h[0] only, the others dim components
  const double g0 = g_h[0];
  const double g1 = mode == AFEM_FACE_SCALAR ? 0.0 : g_h[1];
  const double g2 = (mode == AFEM_FACE_SCALAR || dim == 2) ? 0.0 : g_h[2];
  if (st == AFEM_OK)
    st = launch(ctx, k_face_terms, grid_for(ctx, nb_face, 256), 256, 0, dim, nb_face, coords_d, face_nodes_d,
                outward_d, mode, g0, g1, g2, term);
  if (st == AFEM_OK)
    st = launch(ctx, k_face_gather, grid_for(ctx, nb_node, 256), 256, 0, nb_node, (const int32_t*)ptr,
                (const int32_t*)face, (const double*)term, mode == AFEM_FACE_VECTOR ? dim : 1, nb_dof, rhs_d);
  release();
  return st;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free variant of afem_assemble_poisson_p1.
//
// Some callers cannot let a library allocate device memory while they
// assemble: a host framework that manages every device allocation through its
// own pool and forbids any other cudaMalloc, or code that runs while a stream
// is being captured (where allocating on that stream is not allowed).  This
// entry point takes no context and calls no cudaMalloc / cudaFree / library
// routine that allocates: the element rows live in a fixed file-scope device
// array of kNoAllocRows doubles (32 MiB), which every GPU that loads the
// library keeps until the process exits.  The caller still passes all inputs
// and outputs.

namespace afem {

constexpr size_t kNoAllocRows = size_t(1) << 22;   // doubles: 262,144 tetrahedra or 466,033 triangles
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_rows[kNoAllocRows];

// Device address of g_noalloc_rows, looked up once per device (host code
// must not pass the symbol itself: that is a host-side stand-in).
static double* g_noalloc_addr[kNoAllocMaxDevices] = {};
static std::mutex g_noalloc_mutex;

static afem_status noalloc_rows_address(int dev, double** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_rows);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_rows)", __FILE__, __LINE__);
    g_noalloc_addr[dev] = static_cast<double*>(p);
  }
  *out = g_noalloc_addr[dev];
  return AFEM_OK;
}

template <class Kernel, class... Args>
static afem_status launch_on(cudaStream_t s, Kernel k, unsigned grid, unsigned block, Args... args) {
  // an error left by the caller's own earlier CUDA work is reported as such,
  // not as a failure of this launch
  const cudaError_t pending = cudaPeekAtLastError();
  if (pending != cudaSuccess)
    return cuda_fail(pending, "error pending before the launch (from earlier CUDA work of the caller)", __FILE__,
                     __LINE__);
  k<<<grid, block, 0, s>>>(args...);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? AFEM_OK : cuda_fail(e, "kernel launch", __FILE__, __LINE__);
}

}  // namespace afem

extern "C" afem_status afem_assemble_poisson_p1_noalloc(void* cuda_stream, const afem_mesh_view* m,
                                                        const int32_t* row_ptr_d, const double* cell_coeff_d,
                                                        double* values_d) {
  gather_attrs();
  AFEM_TRY(check_assembly(m, "afem_assemble_poisson_p1_noalloc"));
  AFEM_CHECK_ARG(row_ptr_d && values_d, "afem_assemble_poisson_p1_noalloc: null buffer");
  const size_t npc = m->dim + 1;
  const size_t need = npc * npc * (size_t)m->nb_cell;
  if (need > kNoAllocRows)
    return fail(AFEM_ERR_BAD_ARG,
                "afem_assemble_poisson_p1_noalloc: %d cells need %zu doubles of element rows, above the fixed "
                "%zu (at most %zu tetrahedra or %zu triangles); use afem_assemble_poisson_p1",
                m->nb_cell, need, kNoAllocRows, kNoAllocRows / 16, kNoAllocRows / 9);
  int dev = 0, sms = 0, stream_dev = 0;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(cuda_stream);
  AFEM_CUDA(cudaGetDevice(&dev));
  AFEM_CUDA(cudaStreamGetDevice(s, &stream_dev));
  AFEM_CHECK_ARG(stream_dev == dev,
                 "afem_assemble_poisson_p1_noalloc: cuda_stream belongs to device %d while device %d is current; "
                 "make the stream's device current",
                 stream_dev, dev);
  AFEM_CHECK_ARG(dev >= 0 && dev < kNoAllocMaxDevices, "afem_assemble_poisson_p1_noalloc: device %d unsupported", dev);
  AFEM_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double* rows = nullptr;
  AFEM_TRY(noalloc_rows_address(dev, &rows));
  // every element row is rewritten by the element kernel before the gather
  // reads it, so nothing left by a previous call needs clearing
  // the element rows in the reference's rounding (AFEM_FORMULATION_REFERENCE,
  // the default of a context); no context, so no degenerate-cell flag
  const int64_t eblocks = ((int64_t)m->nb_cell + 127) / 128;
  const unsigned ge = (unsigned)std::max<int64_t>(1, std::min<int64_t>(eblocks, (int64_t)sms * 32));
  const unsigned gg = (unsigned)((m->nb_node + kGatherBlock - 1) / kGatherBlock);
  int* no_flags = nullptr;
  if (m->dim == 3) {
    AFEM_TRY(launch_on(s, k_elem_poisson_p1_ref<4, AFEM_FORMULATION_REFERENCE>, ge, 128, 0, m->nb_cell, m->coords_d,
                       m->cell_nodes_d, m->nc_inverse_d, cell_coeff_d, rows, no_flags));
    return launch_on(s, k_gather_scalar<4>, gg, kGatherBlock, 0, m->nb_node, m->nc_ptr_d, m->nc_slot_d, row_ptr_d,
                     (const double*)rows, values_d);
  }
  AFEM_TRY(launch_on(s, k_elem_poisson_p1_ref<3, AFEM_FORMULATION_REFERENCE>, ge, 128, 0, m->nb_cell, m->coords_d,
                     m->cell_nodes_d, m->nc_inverse_d, cell_coeff_d, rows, no_flags));
  return launch_on(s, k_gather_scalar<3>, gg, kGatherBlock, 0, m->nb_node, m->nc_ptr_d, m->nc_slot_d, row_ptr_d,
                   (const double*)rows, values_d);
}
