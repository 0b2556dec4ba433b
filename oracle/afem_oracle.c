/*
 * afem_oracle.c -- CPU restatement of ArcaneFEM's node-wise P1 path.
 *
 * TEST INFRASTRUCTURE ONLY (the checker, never the product): loaded by
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs.
 *
 * Built with -O2 -ffp-contract=off so that a*b+c is never fused, keeping the
 * reference's operation order and rounding (the reference's CPU build on
 * x86-64 has no FMA contraction).
 */
#include "afem_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

double afo_wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int afo_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* Connectivity                                                              */
/* ------------------------------------------------------------------------ */

/* Arcane's nodeCell() connectivity lists the cells of a node by increasing
 * local id (cells are appended in creation order), used at
 * femutils/BSRFormat.h:428 and modules/testlab/NodeWiseCsrBiliAssembly.cc:188.
 * A counting sort over the cell loop reproduces that order. */
int afo_node_cell(int nb_node, int nb_cell, int npc, const int32_t* cell_nodes, int32_t* nc_ptr,
                  int32_t* nc_cell, uint8_t* nc_local) {
  memset(nc_ptr, 0, sizeof(int32_t) * ((size_t)nb_node + 1));
  for (int64_t k = 0; k < (int64_t)nb_cell * npc; ++k) {
    int32_t n = cell_nodes[k];
    if (n < 0 || n >= nb_node) return -1;
    nc_ptr[n + 1]++;
  }
  for (int i = 0; i < nb_node; ++i) nc_ptr[i + 1] += nc_ptr[i];
  int32_t* cursor = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nb_node > 0 ? nb_node : 1));
  memcpy(cursor, nc_ptr, sizeof(int32_t) * (size_t)nb_node);
  for (int c = 0; c < nb_cell; ++c) {
    for (int l = 0; l < npc; ++l) {
      int32_t n = cell_nodes[(int64_t)c * npc + l];
      int32_t p = cursor[n]++;
      nc_cell[p] = c;
      if (nc_local) nc_local[p] = (uint8_t)l;
    }
  }
  free(cursor);
  return 0;
}

/* BSRFormat::pack (femutils/BSRFormat.h:180-185). */
static uint64_t afo_pack(int32_t n0, int32_t n1) {
  int32_t mn = n0 > n1 ? n1 : n0;
  int32_t mx = n0 > n1 ? n0 : n1;
  return ((uint64_t)(uint32_t)mn << 32) | (uint64_t)(uint32_t)mx;
}

static int cmp_u64(const void* a, const void* b) {
  uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
  return (x > y) - (x < y);
}
static int cmp_i32(const void* a, const void* b) {
  int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
  return (x > y) - (x < y);
}

/* computeSortedEdges / computeNeighbors / computeRowIndex / computeColumns
 * (femutils/BSRFormat.cc:799-971).  The reference fills columns with atomic
 * offsets (:929-971), so its within-row order is not deterministic; rows are
 * sorted here into the canonical order the caller asks for. */
int64_t afo_sparsity(int nb_node, int nb_cell, int npc, const int32_t* cell_nodes, int self_last, int32_t* row_ptr,
                     int32_t* cols, int64_t cap) {
  int pairs = npc * (npc - 1) / 2;
  int64_t nb_edge_total = (int64_t)nb_cell * pairs;
  uint64_t* edges = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)(nb_edge_total > 0 ? nb_edge_total : 1));
  for (int c = 0; c < nb_cell; ++c) {
    const int32_t* cn = cell_nodes + (int64_t)c * npc;
    int64_t start = (int64_t)c * pairs;
    int p = 0;
    for (int i = 0; i < npc; ++i)
      for (int j = i + 1; j < npc; ++j) edges[start + p++] = afo_pack(cn[i], cn[j]);
  }
  qsort(edges, (size_t)nb_edge_total, sizeof(uint64_t), cmp_u64);
  /* neighbours: 1 (self) + unique edges touching the node (:890-924) */
  int32_t* nb = (int32_t*)malloc(sizeof(int32_t) * (size_t)(nb_node > 0 ? nb_node : 1));
  for (int i = 0; i < nb_node; ++i) nb[i] = 1;
  for (int64_t t = 0; t < nb_edge_total; ++t) {
    if (t == nb_edge_total - 1 || edges[t] != edges[t + 1]) {
      int32_t n0 = (int32_t)(edges[t] >> 32), n1 = (int32_t)(edges[t] & 0xFFFFFFFFu);
      nb[n0]++;
      nb[n1]++;
    }
  }
  row_ptr[0] = 0;
  for (int i = 0; i < nb_node; ++i) row_ptr[i + 1] = row_ptr[i] + nb[i];
  int64_t nnz = row_ptr[nb_node];
  if (nnz > cap) {
    free(edges);
    free(nb);
    return -1;
  }
  for (int i = 0; i < nb_node; ++i) nb[i] = 1;
  for (int i = 0; i < nb_node; ++i) cols[row_ptr[i]] = i;
  for (int64_t t = 0; t < nb_edge_total; ++t) {
    if (t == nb_edge_total - 1 || edges[t] != edges[t + 1]) {
      int32_t n0 = (int32_t)(edges[t] >> 32), n1 = (int32_t)(edges[t] & 0xFFFFFFFFu);
      cols[row_ptr[n0] + nb[n0]++] = n1;
      cols[row_ptr[n1] + nb[n1]++] = n0;
    }
  }
  for (int i = 0; i < nb_node; ++i) {
    int32_t b = row_ptr[i], e = row_ptr[i + 1];
    if (self_last) {
      /* neighbours (after the self entry at the row start) ascending, self last */
      qsort(cols + b + 1, (size_t)(e - b - 1), sizeof(int32_t), cmp_i32);
      for (int32_t k = b; k < e - 1; ++k) cols[k] = cols[k + 1];
      cols[e - 1] = i;
    } else {
      qsort(cols + b, (size_t)(e - b), sizeof(int32_t), cmp_i32);
    }
  }
  free(edges);
  free(nb);
  return nnz;
}

/* Node-wise sparsity for the all-core CPU baseline: rows in parallel, each
 * the sorted distinct nodes of the row node's incident cells (self included),
 * the atomic-free construction of femutils/BSRFormat.cc:445-557 with
 * ascending columns.  Two passes (lengths, then columns) around a scan. */
static int row_candidates(int node, int npc, const int32_t* cell_nodes, const int32_t* nc_ptr,
                          const int32_t* nc_cell, int32_t* buf) {
  int m = 0;
  for (int32_t p = nc_ptr[node]; p < nc_ptr[node + 1]; ++p) {
    const int32_t* cn = cell_nodes + (int64_t)nc_cell[p] * npc;
    for (int j = 0; j < npc; ++j) buf[m++] = cn[j];
  }
  buf[m++] = node;   /* a node in no cell keeps its diagonal */
  qsort(buf, (size_t)m, sizeof(int32_t), cmp_i32);
  int u = 0;
  for (int k = 0; k < m; ++k)
    if (k == 0 || buf[k] != buf[k - 1]) buf[u++] = buf[k];
  return u;
}

int64_t afo_sparsity_nodewise(int nb_node, int npc, const int32_t* cell_nodes, const int32_t* nc_ptr,
                              const int32_t* nc_cell, int32_t* row_ptr, int32_t* cols, int64_t cap,
                              int nb_threads) {
  int maxdeg = 0;
  for (int i = 0; i < nb_node; ++i)
    if (nc_ptr[i + 1] - nc_ptr[i] > maxdeg) maxdeg = nc_ptr[i + 1] - nc_ptr[i];
  const size_t bufsz = (size_t)maxdeg * npc + 1;
  if (nb_threads < 1) nb_threads = 1;
  row_ptr[0] = 0;
#ifdef _OPENMP
#pragma omp parallel num_threads(nb_threads)
#endif
  {
    int32_t* buf = (int32_t*)malloc(sizeof(int32_t) * bufsz);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int i = 0; i < nb_node; ++i) row_ptr[i + 1] = row_candidates(i, npc, cell_nodes, nc_ptr, nc_cell, buf);
    free(buf);
  }
  for (int i = 0; i < nb_node; ++i) row_ptr[i + 1] += row_ptr[i];
  if (row_ptr[nb_node] > cap) return -1;
#ifdef _OPENMP
#pragma omp parallel num_threads(nb_threads)
#endif
  {
    int32_t* buf = (int32_t*)malloc(sizeof(int32_t) * bufsz);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int i = 0; i < nb_node; ++i) {
      const int u = row_candidates(i, npc, cell_nodes, nc_ptr, nc_cell, buf);
      memcpy(cols + row_ptr[i], buf, sizeof(int32_t) * (size_t)u);
    }
    free(buf);
  }
  return row_ptr[nb_node];
}

/* ------------------------------------------------------------------------ */
/* Geometry (femutils/ArcaneFemFunctionsGpu.h)                               */
/* ------------------------------------------------------------------------ */

typedef struct { double x, y, z; } r3;

static r3 node(const double* coords, int32_t n) {
  r3 r = {coords[3 * (int64_t)n], coords[3 * (int64_t)n + 1], coords[3 * (int64_t)n + 2]};
  return r;
}
static r3 sub3(r3 a, r3 b) { r3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static r3 cross3(r3 a, r3 b) {
  r3 r = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
  return r;
}
static double dot3(r3 a, r3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

/* computeAreaTria3 (ArcaneFemFunctionsGpu.h:76-86): |cross(n1-n0, n2-n0)| / 2 */
static double area_tria3(const double* coords, const int32_t* cn) {
  r3 n0 = node(coords, cn[0]), n1 = node(coords, cn[1]), n2 = node(coords, cn[2]);
  r3 v = cross3(sub3(n1, n0), sub3(n2, n0));
  return sqrt(v.x * v.x + v.y * v.y + v.z * v.z) / 2.0;
}

/* computeVolumeTetra4 (ArcaneFemFunctionsGpu.h:113-128) */
static double volume_tetra4(const double* coords, const int32_t* cn) {
  r3 n0 = node(coords, cn[0]), n1 = node(coords, cn[1]), n2 = node(coords, cn[2]), n3 = node(coords, cn[3]);
  r3 v0 = sub3(n1, n0), v1 = sub3(n2, n0), v2 = sub3(n3, n0);
  return fabs(dot3(v0, cross3(v1, v2))) / 6.0;
}

/* computeGradientXTria3 / computeGradientYTria3 (ArcaneFemFunctionsGpu.h:241-281) */
static void grad_tria3(const double* coords, const int32_t* cn, double dx[3], double dy[3]) {
  r3 n0 = node(coords, cn[0]), n1 = node(coords, cn[1]), n2 = node(coords, cn[2]);
  double A2 = ((n1.x - n0.x) * (n2.y - n0.y) - (n2.x - n0.x) * (n1.y - n0.y));
  dx[0] = (n1.y - n2.y) / A2;
  dx[1] = (n2.y - n0.y) / A2;
  dx[2] = (n0.y - n1.y) / A2;
  dy[0] = (n2.x - n1.x) / A2;
  dy[1] = (n0.x - n2.x) / A2;
  dy[2] = (n1.x - n0.x) / A2;
}

/* computeGradient{X,Y,Z}Tetra4 (ArcaneFemFunctionsGpu.h:414-535) */
static void grad_tetra4(const double* coords, const int32_t* cn, double dx[4], double dy[4], double dz[4]) {
  r3 n0 = node(coords, cn[0]), n1 = node(coords, cn[1]), n2 = node(coords, cn[2]), n3 = node(coords, cn[3]);
  r3 v0 = sub3(n1, n0), v1 = sub3(n2, n0), v2 = sub3(n3, n0);
  double V6 = fabs(dot3(v0, cross3(v1, v2)));
  dx[0] = (n1.y * (n3.z - n2.z) + n2.y * (n1.z - n3.z) + n3.y * (n2.z - n1.z)) / V6;
  dx[1] = (n0.y * (n2.z - n3.z) + n2.y * (n3.z - n0.z) + n3.y * (n0.z - n2.z)) / V6;
  dx[2] = (n0.y * (n3.z - n1.z) + n1.y * (n0.z - n3.z) + n3.y * (n1.z - n0.z)) / V6;
  dx[3] = (n0.y * (n1.z - n2.z) + n1.y * (n2.z - n0.z) + n2.y * (n0.z - n1.z)) / V6;
  dy[0] = (n1.z * (n3.x - n2.x) + n2.z * (n1.x - n3.x) + n3.z * (n2.x - n1.x)) / V6;
  dy[1] = (n0.z * (n2.x - n3.x) + n2.z * (n3.x - n0.x) + n3.z * (n0.x - n2.x)) / V6;
  dy[2] = (n0.z * (n3.x - n1.x) + n1.z * (n0.x - n3.x) + n3.z * (n1.x - n0.x)) / V6;
  dy[3] = (n0.z * (n1.x - n2.x) + n1.z * (n2.x - n0.x) + n2.z * (n0.x - n1.x)) / V6;
  dz[0] = (n1.x * (n3.y - n2.y) + n2.x * (n1.y - n3.y) + n3.x * (n2.y - n1.y)) / V6;
  dz[1] = (n0.x * (n2.y - n3.y) + n2.x * (n3.y - n0.y) + n3.x * (n0.y - n2.y)) / V6;
  dz[2] = (n0.x * (n3.y - n1.y) + n1.x * (n0.y - n3.y) + n3.x * (n1.y - n0.y)) / V6;
  dz[3] = (n0.x * (n1.y - n2.y) + n1.x * (n2.y - n0.y) + n2.x * (n0.y - n1.y)) / V6;
}

/* ------------------------------------------------------------------------ */
/* Element row vectors                                                       */
/* ------------------------------------------------------------------------ */

/* _computeElementVectorTria3Gpu (modules/poisson/ElementMatrix.h:54-63):
 *   area * dxU[i] * dxU + area * dyU[i] * dyU */
void afo_elem_vec_poisson_tri3(const double* coords, const int32_t* cn, int i, double out[3]) {
  double area = area_tria3(coords, cn);
  double dx[3], dy[3];
  grad_tria3(coords, cn, dx, dy);
  double sx = area * dx[i], sy = area * dy[i];
  for (int k = 0; k < 3; ++k) out[k] = sx * dx[k] + sy * dy[k];
}

/* _computeElementVectorTetra4Gpu (modules/poisson/ElementMatrix.h:107-118) */
void afo_elem_vec_poisson_tet4(const double* coords, const int32_t* cn, int i, double out[4]) {
  double vol = volume_tetra4(coords, cn);
  double dx[4], dy[4], dz[4];
  grad_tetra4(coords, cn, dx, dy, dz);
  double sx = vol * dx[i], sy = vol * dy[i], sz = vol * dz[i];
  for (int k = 0; k < 4; ++k) out[k] = sx * dx[k] + sy * dy[k] + sz * dz[k];
}

/* _computeCellMatrixGpuTRIA3 (modules/testlab/FemModule.h:469-495) and the row
 * loop of _assembleNodeWiseCsrBilinearOperatorTria3
 * (modules/testlab/NodeWiseCsrBiliAssembly.cc:194-211): x = B_i . B_j; x * area
 * with the signed area. */
void afo_elem_vec_testlab_tri3(const double* coords, const int32_t* cn, int i, double out[3]) {
  r3 m0 = node(coords, cn[0]), m1 = node(coords, cn[1]), m2 = node(coords, cn[2]);
  double area = 0.5 * ((m1.x - m0.x) * (m2.y - m0.y) - (m2.x - m0.x) * (m1.y - m0.y));
  double p[3][2] = {{m1.y - m2.y, m2.x - m1.x}, {m2.y - m0.y, m0.x - m2.x}, {m0.y - m1.y, m1.x - m0.x}};
  double mul = 0.5 / area;
  double b[6];
  for (int k = 0; k < 3; ++k) {
    b[2 * k] = p[k][0] * mul;
    b[2 * k + 1] = p[k][1] * mul;
  }
  for (int k = 0; k < 3; ++k) {
    double x = b[i * 2] * b[k * 2] + b[i * 2 + 1] * b[k * 2 + 1];
    out[k] = x * area;
  }
}

/* _computeCellMatrixGpuTETRA4 (modules/testlab/FemModule.h:498-538) and the
 * row loop of _assembleNodeWiseCsrBilinearOperatorTetra4
 * (NodeWiseCsrBiliAssembly.cc:269-290). */
void afo_elem_vec_testlab_tet4(const double* coords, const int32_t* cn, int i, double out[4]) {
  r3 m0 = node(coords, cn[0]), m1 = node(coords, cn[1]), m2 = node(coords, cn[2]), m3 = node(coords, cn[3]);
  r3 v0 = sub3(m1, m0), v1 = sub3(m2, m0), v2 = sub3(m3, m0);
  double volume = fabs(dot3(v0, cross3(v1, v2))) / 6.0;
  r3 d[4];
  d[0] = cross3(sub3(m2, m1), sub3(m1, m3));
  d[1] = cross3(sub3(m3, m0), sub3(m0, m2));
  d[2] = cross3(sub3(m1, m0), sub3(m0, m3));
  d[3] = cross3(sub3(m0, m1), sub3(m1, m2));
  double mul = 1.0 / (6.0 * volume);
  double b[12];
  for (int k = 0; k < 4; ++k) {
    b[3 * k] = d[k].x * mul;
    b[3 * k + 1] = d[k].y * mul;
    b[3 * k + 2] = d[k].z * mul;
  }
  for (int k = 0; k < 4; ++k) {
    double x = b[i * 3] * b[k * 3] + b[i * 3 + 1] * b[k * 3 + 1] + b[i * 3 + 2] * b[k * 3 + 2];
    out[k] = x * volume;
  }
}

/* computeElementVectorTetra4Gpu (modules/elasticity/ElementMatrix.h:216-301),
 * restated with the same 12-vectors (zeros included) and the same order:
 *   (lambda + 2 mu) * ( a*dxUx + b*dyUy + c*dzUz ) * volume, etc.
 * out is row-major [3][12]. */
void afo_elem_vec_elasticity_tet4(const double* coords, const int32_t* cn, double lambda, double mu, int nl,
                                  double out[36]) {
  double dxu[4], dyu[4], dzu[4];
  grad_tetra4(coords, cn, dxu, dyu, dzu);
  double volume = volume_tetra4(coords, cn);
  double dxUx[12] = {0}, dyUx[12] = {0}, dzUx[12] = {0};
  double dxUy[12] = {0}, dyUy[12] = {0}, dzUy[12] = {0};
  double dxUz[12] = {0}, dyUz[12] = {0}, dzUz[12] = {0};
  for (int n = 0; n < 4; ++n) {
    dxUx[3 * n] = dxu[n]; dyUx[3 * n] = dyu[n]; dzUx[3 * n] = dzu[n];
    dxUy[3 * n + 1] = dxu[n]; dyUy[3 * n + 1] = dyu[n]; dzUy[3 * n + 1] = dzu[n];
    dxUz[3 * n + 2] = dxu[n]; dyUz[3 * n + 2] = dyu[n]; dzUz[3 * n + 2] = dzu[n];
  }
  double l2m = lambda + 2 * mu;
  for (int a = 0; a < 3; ++a) {
    int r = nl * 3 + a;
    for (int k = 0; k < 12; ++k) {
      /* normal strain energy */
      double ne = l2m * (((dxUx[r] * dxUx[k]) + (dyUy[r] * dyUy[k])) + (dzUz[r] * dzUz[k])) * volume;
      /* compressibility effect */
      double ce = lambda *
                  (((((dyUy[r] * dxUx[k]) + (dxUx[r] * dyUy[k])) + (dzUz[r] * dxUx[k])) + (dxUx[r] * dzUz[k])) +
                    (dyUy[r] * dzUz[k]) + (dzUz[r] * dyUy[k])) *
                  volume;
      /* shear energy */
      double se = mu *
                  ((((dxUy[r] + dyUx[r]) * (dyUx[k] + dxUy[k])) + ((dzUy[r] + dyUz[r]) * (dyUz[k] + dzUy[k]))) +
                   ((dxUz[r] + dzUx[r]) * (dzUx[k] + dxUz[k]))) *
                  volume;
      out[a * 12 + k] = ne + ce + se;
    }
  }
}

/* _computeElementVectorQuad4Gpu (modules/poisson/ElementMatrixHexQuad.h:63-91)
 * with computeGradientsAndJacobianQuad4Gpu (femutils/ArcaneFemFunctionsGpu.h:
 * 298-360) and computeReferenceGradientsQuad4 (femutils/ShapeFunctions.h:123-129). */
static const double kGp = 0.57735026918962576451;
void afo_elem_vec_poisson_quad4(const double* coords, const int32_t* cn, int i, double out[4]) {
  const double gp[2] = {-kGp, kGp};
  for (int k = 0; k < 4; ++k) out[k] = 0.0;
  for (int ixi = 0; ixi < 2; ++ixi)
    for (int ieta = 0; ieta < 2; ++ieta) {
      const double xi = gp[ixi], eta = gp[ieta];
      const double dxi[4] = {-0.25 * (1.0 - eta), 0.25 * (1.0 - eta), 0.25 * (1.0 + eta), -0.25 * (1.0 + eta)};
      const double deta[4] = {-0.25 * (1.0 - xi), -0.25 * (1.0 + xi), 0.25 * (1.0 + xi), 0.25 * (1.0 - xi)};
      double J00 = 0.0, J01 = 0.0, J10 = 0.0, J11 = 0.0;
      for (int a = 0; a < 4; ++a) {
        const double* c = coords + 3 * (int64_t)cn[a];
        J00 += dxi[a] * c[0];
        J01 += dxi[a] * c[1];
        J10 += deta[a] * c[0];
        J11 += deta[a] * c[1];
      }
      const double detJ = J00 * J11 - J01 * J10;
      const double invJ00 = J11 / detJ, invJ01 = -J01 / detJ, invJ10 = -J10 / detJ, invJ11 = J00 / detJ;
      double dx[4], dy[4];
      for (int a = 0; a < 4; ++a) {
        dx[a] = invJ00 * dxi[a] + invJ01 * deta[a];
        dy[a] = invJ10 * dxi[a] + invJ11 * deta[a];
      }
      const double w = detJ * 1.0 * 1.0;
      for (int k = 0; k < 4; ++k) out[k] += (dx[i] * dx[k]) * w + (dy[i] * dy[k]) * w;
    }
}

/* _computeElementVectorHexa8Gpu (modules/poisson/ElementMatrixHexQuad.h:239-266)
 * with _computeHexaGradientsAndJacobian (femutils/ArcaneFemFunctionsGpu.h:
 * 554-586) and computeReferenceGradientsHexa8 (femutils/ShapeFunctions.h:
 * 314-345).  Arcane's math::matrixDeterminant / inverseMatrix (not in the
 * reference tree) are restated as the expansion along the first row and the
 * adjugate divided by the determinant. */
void afo_elem_vec_poisson_hexa8(const double* coords, const int32_t* cn, int i, double out[8]) {
  const double gp[2] = {-kGp, kGp};
  for (int k = 0; k < 8; ++k) out[k] = 0.0;
  for (int ixi = 0; ixi < 2; ++ixi)
    for (int ieta = 0; ieta < 2; ++ieta)
      for (int izeta = 0; izeta < 2; ++izeta) {
        const double xi = gp[ixi], eta = gp[ieta], zeta = gp[izeta];
        const double dxi[8] = {-0.125 * (1.0 - eta) * (1.0 - zeta), 0.125 * (1.0 - eta) * (1.0 - zeta),
                               0.125 * (1.0 + eta) * (1.0 - zeta),  -0.125 * (1.0 + eta) * (1.0 - zeta),
                               -0.125 * (1.0 - eta) * (1.0 + zeta), 0.125 * (1.0 - eta) * (1.0 + zeta),
                               0.125 * (1.0 + eta) * (1.0 + zeta),  -0.125 * (1.0 + eta) * (1.0 + zeta)};
        const double deta[8] = {-0.125 * (1.0 - xi) * (1.0 - zeta), -0.125 * (1.0 + xi) * (1.0 - zeta),
                                0.125 * (1.0 + xi) * (1.0 - zeta),  0.125 * (1.0 - xi) * (1.0 - zeta),
                                -0.125 * (1.0 - xi) * (1.0 + zeta), -0.125 * (1.0 + xi) * (1.0 + zeta),
                                0.125 * (1.0 + xi) * (1.0 + zeta),  0.125 * (1.0 - xi) * (1.0 + zeta)};
        const double dzeta[8] = {-0.125 * (1.0 - xi) * (1.0 - eta), -0.125 * (1.0 + xi) * (1.0 - eta),
                                 -0.125 * (1.0 + xi) * (1.0 + eta), -0.125 * (1.0 - xi) * (1.0 + eta),
                                 0.125 * (1.0 - xi) * (1.0 - eta),  0.125 * (1.0 + xi) * (1.0 - eta),
                                 0.125 * (1.0 + xi) * (1.0 + eta),  0.125 * (1.0 - xi) * (1.0 + eta)};
        double J[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
        for (int a = 0; a < 8; ++a) {
          const double* c = coords + 3 * (int64_t)cn[a];
          for (int d = 0; d < 3; ++d) {
            J[0][d] += dxi[a] * c[d];
            J[1][d] += deta[a] * c[d];
            J[2][d] += dzeta[a] * c[d];
          }
        }
        const double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                           J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                           J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        double inv[3][3];
        inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det;
        inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
        inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det;
        inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
        inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det;
        inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
        inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det;
        inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
        inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
        double dx[8], dy[8], dz[8];
        for (int a = 0; a < 8; ++a) {
          dx[a] = inv[0][0] * dxi[a] + inv[0][1] * deta[a] + inv[0][2] * dzeta[a];
          dy[a] = inv[1][0] * dxi[a] + inv[1][1] * deta[a] + inv[1][2] * dzeta[a];
          dz[a] = inv[2][0] * dxi[a] + inv[2][1] * deta[a] + inv[2][2] * dzeta[a];
        }
        for (int k = 0; k < 8; ++k) {
          const double grad_dot = dx[i] * dx[k] + dy[i] * dy[k] + dz[i] * dz[k];
          out[k] += grad_dot * det;
        }
      }
}

/* ------------------------------------------------------------------------ */
/* Node-wise assembly                                                        */
/* ------------------------------------------------------------------------ */

static int kind_npc(int kind) {
  if (kind == AFO_POISSON_QUAD4) return 4;
  if (kind == AFO_POISSON_HEXA8) return 8;
  return (kind == AFO_POISSON_TRI3 || kind == AFO_TESTLAB_TRI3) ? 3 : 4;
}
static int kind_block(int kind) { return kind == AFO_ELASTICITY_TET4 ? 3 : 1; }

/* assembleBilinearOrderedPerBlockAtomicFree (femutils/BSRFormat.h:406-470) and
 * assembleBilinearOrderedPerRowAtomicFree (BSRFormat.h:473-537). */
int afo_assemble_nodewise(int kind, int nb_node, int nb_cell, const double* coords, const int32_t* cell_nodes,
                          const int32_t* nc_ptr, const int32_t* nc_cell, const int32_t* row_ptr,
                          const int32_t* cols, int per_block_layout, double lambda, double mu,
                          const double* cell_coeff, double* values, int nb_threads) {
  (void)nb_cell;
  const int npc = kind_npc(kind);
  const int b = kind_block(kind);
  const int bb = b * b;
  int bad = 0;
#ifdef _OPENMP
  if (nb_threads < 1) nb_threads = 1;
#pragma omp parallel for schedule(static) num_threads(nb_threads) reduction(| : bad)
#endif
  for (int row = 0; row < nb_node; ++row) {
    for (int32_t p = nc_ptr[row]; p < nc_ptr[row + 1]; ++p) {
      int32_t cell = nc_cell[p];
      const int32_t* cn = cell_nodes + (int64_t)cell * npc;
      int li = -1;
      for (int i = 0; i < npc; ++i)
        if (cn[i] == row) { li = i; break; }
      if (li < 0) continue;
      double ev[36];
      switch (kind) {
        case AFO_POISSON_TRI3: afo_elem_vec_poisson_tri3(coords, cn, li, ev); break;
        case AFO_POISSON_TET4: afo_elem_vec_poisson_tet4(coords, cn, li, ev); break;
        case AFO_TESTLAB_TRI3: afo_elem_vec_testlab_tri3(coords, cn, li, ev); break;
        case AFO_TESTLAB_TET4: afo_elem_vec_testlab_tet4(coords, cn, li, ev); break;
        case AFO_POISSON_QUAD4: afo_elem_vec_poisson_quad4(coords, cn, li, ev); break;
        case AFO_POISSON_HEXA8: afo_elem_vec_poisson_hexa8(coords, cn, li, ev); break;
        default: afo_elem_vec_elasticity_tet4(coords, cn, lambda, mu, li, ev); break;
      }
      double coeff = cell_coeff ? cell_coeff[cell] : 1.0;
      int32_t begin0 = row_ptr[row], end = row_ptr[row + 1];
      int32_t nnzb_row = end - begin0;
      for (int j = 0; j < npc; ++j) {
        int32_t col = cn[j];
        int found = 0;
        for (int32_t x = 0, k = begin0; k < end; ++k, ++x) {
          if (cols[k] != col) continue;
          for (int bi = 0; bi < b; ++bi)
            for (int bj = 0; bj < b; ++bj) {
              double v = ev[bi * (b * npc) + b * j + bj];
              if (cell_coeff) v = coeff * v;
              int64_t idx = per_block_layout ? (int64_t)k * bb + bi * b + bj
                                             : (int64_t)begin0 * bb + (int64_t)b * (x + bi * nnzb_row) + bj;
              values[idx] += v;
            }
          found = 1;
          break;
        }
        if (!found) bad = 1;
      }
    }
  }
  return bad ? -1 : 0;
}

/* ------------------------------------------------------------------------ */
/* Right-hand side and boundary conditions                                  */
/* ------------------------------------------------------------------------ */

/* applyConstantSourceToRhsBase (femutils/ArcaneFemFunctionsGpu.h:676-708):
 *   sum += qdot * domain / nb_node_of_cell;  rhs[dof(node,0)] = sum */
void afo_rhs_constant_source(int dim, int nb_node, const double* coords, const int32_t* cell_nodes, int npc,
                             const int32_t* nc_ptr, const int32_t* nc_cell, double qdot, int nb_dof,
                             double* rhs) {
  for (int n = 0; n < nb_node; ++n) {
    double sum = 0.0;
    for (int32_t p = nc_ptr[n]; p < nc_ptr[n + 1]; ++p) {
      const int32_t* cn = cell_nodes + (int64_t)nc_cell[p] * npc;
      double domain = dim == 2 ? area_tria3(coords, cn) : volume_tetra4(coords, cn);
      sum += qdot * domain / npc;
    }
    rhs[(int64_t)n * nb_dof] = sum;
  }
}

/* applyConstantSourceToRhsQuad4 / Hexa8 (femutils/ArcaneFemFunctionsGpu.cc:
 * 393-458,875-960): N_i qdot (w detJ) per Gauss point, summed per node over
 * its cells in increasing order (the reference's atomics have no fixed order). */
void afo_rhs_constant_source_q1(int dim, int nb_node, const double* coords, const int32_t* cell_nodes,
                                const int32_t* nc_ptr, const int32_t* nc_cell, double qdot, int nb_dof,
                                double* rhs) {
  const int npc = 1 << dim;
  const double gp[2] = {-kGp, kGp};
  for (int n = 0; n < nb_node; ++n) {
    double sum = 0.0;
    for (int32_t p = nc_ptr[n]; p < nc_ptr[n + 1]; ++p) {
      const int32_t* cn = cell_nodes + (int64_t)nc_cell[p] * npc;
      int li = 0;
      while (cn[li] != n) ++li;
      for (int ixi = 0; ixi < 2; ++ixi)
        for (int ieta = 0; ieta < 2; ++ieta)
          for (int izeta = 0; izeta < (dim == 3 ? 2 : 1); ++izeta) {
            const double xi = gp[ixi], eta = gp[ieta], zeta = gp[izeta];
            double Ni, detJ;
            if (dim == 2) {
              const double Nq[4] = {0.25 * (1.0 - xi) * (1.0 - eta), 0.25 * (1.0 + xi) * (1.0 - eta),
                                    0.25 * (1.0 + xi) * (1.0 + eta), 0.25 * (1.0 - xi) * (1.0 + eta)};
              const double dxi[4] = {-0.25 * (1.0 - eta), 0.25 * (1.0 - eta), 0.25 * (1.0 + eta), -0.25 * (1.0 + eta)};
              const double deta[4] = {-0.25 * (1.0 - xi), -0.25 * (1.0 + xi), 0.25 * (1.0 + xi), 0.25 * (1.0 - xi)};
              double J00 = 0.0, J01 = 0.0, J10 = 0.0, J11 = 0.0;
              for (int a = 0; a < 4; ++a) {
                const double* c = coords + 3 * (int64_t)cn[a];
                J00 += dxi[a] * c[0];
                J01 += dxi[a] * c[1];
                J10 += deta[a] * c[0];
                J11 += deta[a] * c[1];
              }
              detJ = J00 * J11 - J01 * J10;
              Ni = Nq[li];
            } else {
              const double mx = 1.0 - xi, px = 1.0 + xi, me = 1.0 - eta, pe = 1.0 + eta, mz = 1.0 - zeta,
                           pz = 1.0 + zeta;
              const double Nh[8] = {0.125 * mx * me * mz, 0.125 * px * me * mz, 0.125 * px * pe * mz,
                                    0.125 * mx * pe * mz, 0.125 * mx * me * pz, 0.125 * px * me * pz,
                                    0.125 * px * pe * pz, 0.125 * mx * pe * pz};
              const double dxi[8] = {-0.125 * me * mz, 0.125 * me * mz, 0.125 * pe * mz, -0.125 * pe * mz,
                                     -0.125 * me * pz, 0.125 * me * pz, 0.125 * pe * pz, -0.125 * pe * pz};
              const double deta[8] = {-0.125 * mx * mz, -0.125 * px * mz, 0.125 * px * mz, 0.125 * mx * mz,
                                      -0.125 * mx * pz, -0.125 * px * pz, 0.125 * px * pz, 0.125 * mx * pz};
              const double dzeta[8] = {-0.125 * mx * me, -0.125 * px * me, -0.125 * px * pe, -0.125 * mx * pe,
                                       0.125 * mx * me, 0.125 * px * me, 0.125 * px * pe, 0.125 * mx * pe};
              double J[3][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
              for (int a = 0; a < 8; ++a) {
                const double* c = coords + 3 * (int64_t)cn[a];
                for (int d = 0; d < 3; ++d) {
                  J[0][d] += dxi[a] * c[d];
                  J[1][d] += deta[a] * c[d];
                  J[2][d] += dzeta[a] * c[d];
                }
              }
              detJ = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                     J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
              Ni = Nh[li];
            }
            sum += Ni * qdot * (1.0 * detJ);
          }
    }
    rhs[(int64_t)n * nb_dof] = sum;
  }
}

/* FemModuleElasticity::_applyBodyForce, tetrahedra (modules/elasticity/BodyForce.h:148-160) */
void afo_rhs_body_force_tet4(int nb_cell, const double* coords, const int32_t* cell_nodes, const double f[3],
                             double* rhs) {
  for (int c = 0; c < nb_cell; ++c) {
    const int32_t* cn = cell_nodes + (int64_t)c * 4;
    double volume = volume_tetra4(coords, cn);
    for (int k = 0; k < 4; ++k) {
      int64_t d = (int64_t)cn[k] * 3;
      rhs[d] += f[0] * volume / 4;
      rhs[d + 1] += f[1] * volume / 4;
      rhs[d + 2] += f[2] * volume / 4;
    }
  }
}

/* Boundary-face terms on P1 meshes, faces in the order given, nodes in face
 * order, += into the right-hand side (the CPU paths' sequential order):
 *   mode 0, scalar Neumann:  rhs[dof(n, 0)] += g0 * |f| / nf
 *     (applyNeumannToRhsTria3 / Tetra4, femutils/ArcaneFemFunctionsGpu.cc:679-735,1082-1140)
 *   mode 1, normal Neumann:  rhs[dof(n, 0)] += (nrm . g) * |f| / nf   (same functions, vector branch)
 *   mode 2, traction:        rhs[dof(n, c)] += g_c * |f| / nf, c < dim
 *     (applyTractionToRhsTria3 / Tetra4, femutils/ArcaneFemFunctions.h:2854-2885,2188-2220)
 * |f|: edge length sqrt(dx dx + dy dy) (ArcaneFemFunctionsGpu.h:139-147) or
 * triangle area |(n1 - n0) x (n2 - n0)| / 2 (:92-102); nrm: the unit outward
 * normal (:159-178, :190-213), the face's first two nodes swapped when the
 * face is not oriented outward (outward[f] == 0).  Arcane's Real3::normL2 is
 * sqrt(x x + y y + z z). */
void afo_rhs_boundary_faces(int dim, int nb_face, const double* coords, const int32_t* face_nodes,
                            const uint8_t* outward, int mode, const double g[3], int nb_dof, double* rhs) {
  const int nf = dim;
  for (int f = 0; f < nb_face; ++f) {
    const int32_t* fn = face_nodes + (int64_t)f * nf;
    const double* a0 = coords + 3 * (int64_t)fn[0];
    const double* a1 = coords + 3 * (int64_t)fn[1];
    double measure, nrm[3] = {0.0, 0.0, 0.0};
    const int out = outward ? outward[f] : 1;
    if (dim == 2) {
      const double dx = a1[0] - a0[0], dy = a1[1] - a0[1];
      measure = sqrt(dx * dx + dy * dy);
      const double* b0 = out ? a0 : a1;
      const double* b1 = out ? a1 : a0;
      const double ex = b1[0] - b0[0], ey = b1[1] - b0[1];
      const double nn = sqrt(ey * ey + ex * ex);
      nrm[0] = ey / nn;
      nrm[1] = (b0[0] - b1[0]) / nn;
    } else {
      const double* a2 = coords + 3 * (int64_t)fn[2];
      const double u[3] = {a1[0] - a0[0], a1[1] - a0[1], a1[2] - a0[2]};
      const double v[3] = {a2[0] - a0[0], a2[1] - a0[1], a2[2] - a0[2]};
      const double c[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
      measure = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) / 2.0;
      const double* b0 = out ? a0 : a1;
      const double* b1 = out ? a1 : a0;
      const double e1[3] = {b1[0] - b0[0], b1[1] - b0[1], b1[2] - b0[2]};
      const double e2[3] = {a2[0] - b0[0], a2[1] - b0[1], a2[2] - b0[2]};
      const double m[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
      const double nn = sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
      nrm[0] = m[0] / nn;
      nrm[1] = m[1] / nn;
      nrm[2] = m[2] / nn;
    }
    for (int k = 0; k < nf; ++k) {
      const int64_t d = (int64_t)fn[k] * nb_dof;
      if (mode == 0) {
        rhs[d] += g[0] * measure / nf;
      } else if (mode == 1) {
        const double flux = dim == 2 ? nrm[0] * g[0] + nrm[1] * g[1] : nrm[0] * g[0] + nrm[1] * g[1] + nrm[2] * g[2];
        rhs[d] += flux * measure / nf;
      } else {
        for (int c = 0; c < dim; ++c) rhs[d + c] += g[c] * measure / nf;
      }
    }
  }
}

/* applyDirichletToNodeGroupViaPenalty (femutils/ArcaneFemFunctionsGpu.cc:54-78) */
void afo_dirichlet_penalty(int nb_sel, const int32_t* nodes, int nb_dof, int dof_index, double value,
                           double penalty, uint8_t* forced_info, double* forced_value, double* rhs) {
  for (int s = 0; s < nb_sel; ++s) {
    int64_t d = (int64_t)nodes[s] * nb_dof + dof_index;
    forced_info[d] = 1;
    forced_value[d] = penalty;
    rhs[d] = penalty * value;
  }
}

/* applyDirichletToNodeGroupViaRowOrRowColumnElimination (ArcaneFemFunctionsGpu.cc:83-105) */
void afo_dirichlet_elimination(int nb_sel, const int32_t* nodes, int nb_dof, int dof_index, double value,
                               uint8_t elimination_type, uint8_t* elim_info, double* elim_value) {
  for (int s = 0; s < nb_sel; ++s) {
    int64_t d = (int64_t)nodes[s] * nb_dof + dof_index;
    elim_info[d] = elimination_type;
    elim_value[d] = value;
  }
}

enum { ELIM_NONE = 0, ELIM_ROW = 1, ELIM_ROW_COLUMN = 2 }; /* femutils/FemUtilsGlobal.h:51-62 */

void afo_apply_matrix_transformation(int nb_row, const int32_t* row_ptr, const int32_t* cols, double* values,
                                     const uint8_t* forced_info, const double* forced_value,
                                     const uint8_t* elim_info, const double* elim_value, double* rc_saved,
                                     uint8_t* rc_mask) {
  (void)elim_value;
  /* _fillRowColumnEliminationInfos (CsrDoFLinearSystemImpl.cc:187-230) */
  int has_rc = 0;
  for (int i = 0; i < nb_row; ++i)
    if (elim_info[i] == ELIM_ROW_COLUMN) { has_rc = 1; break; }
  if (rc_mask) memset(rc_mask, 0, (size_t)row_ptr[nb_row]);
  if (has_rc && rc_saved && rc_mask) {
    for (int i = 0; i < nb_row; ++i)
      for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        int32_t c = cols[k];
        if (c >= 0 && (elim_info[i] == ELIM_ROW_COLUMN || elim_info[c] == ELIM_ROW_COLUMN)) {
          rc_saved[k] = values[k];
          rc_mask[k] = 1;
        }
      }
  }
  /* _applyRowEliminationOnMatrix (:126-152) */
  for (int i = 0; i < nb_row; ++i)
    if (elim_info[i] == ELIM_ROW)
      for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) values[k] = (cols[k] == i) ? 1.0 : 0.0;
  /* _applyRowColumnEliminationOnMatrix (:88-121), including its column_index > 0 test */
  if (has_rc) {
    for (int i = 0; i < nb_row; ++i) {
      int is_row = elim_info[i] == ELIM_ROW || elim_info[i] == ELIM_ROW_COLUMN;
      for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        int32_t c = cols[k];
        if (c > 0) {
          int is_col = elim_info[c] == ELIM_ROW || elim_info[c] == ELIM_ROW_COLUMN;
          if (is_row || is_col) values[k] = (c == i) ? 1.0 : 0.0;
        }
      }
    }
  }
  /* _applyForcedValuesToLhs (:50-72) */
  for (int i = 0; i < nb_row; ++i)
    if (forced_info[i])
      for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k)
        if (cols[k] == i) { values[k] = forced_value[i]; break; }
}

void afo_apply_rhs_transformation(int nb_row, const int32_t* row_ptr, const int32_t* cols, const uint8_t* elim_info,
                                  const double* elim_value, const double* rc_saved, const uint8_t* rc_mask,
                                  double* rhs) {
  /* _applyRowColumnEliminationToRHS (DoFLinearSystemImplBase.cc:55-88): the
   * map is walked in (row, column) order; rhs[col] -= A[row, col] * g[row]
   * for every kept entry whose row is RowColumn-eliminated. */
  if (rc_saved && rc_mask) {
    for (int i = 0; i < nb_row; ++i) {
      if (elim_info[i] != ELIM_ROW_COLUMN) continue;
      for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
        int32_t c = cols[k];
        if (!rc_mask[k] || c == i) continue;
        double v = rhs[c];
        rhs[c] = v - rc_saved[k] * elim_value[i];
      }
    }
  }
  /* _applyRowOrRowColumnEliminationOnRHS (CsrDoFLinearSystemImpl.cc:157-182) */
  for (int i = 0; i < nb_row; ++i)
    if (elim_info[i] == ELIM_ROW || elim_info[i] == ELIM_ROW_COLUMN) rhs[i] = elim_value[i];
}

/* ------------------------------------------------------------------------ */
/* Krylov                                                                    */
/* ------------------------------------------------------------------------ */

void afo_spmv(int nb_row, const int32_t* row_ptr, const int32_t* cols, const double* values, const double* x,
              double* y) {
  for (int i = 0; i < nb_row; ++i) {
    double s = 0.0;
    for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) s += values[k] * x[cols[k]];
    y[i] = s;
  }
}

static double pdot(int n, const double* a, const double* b, int nt) {
  double s = 0.0;
  (void)nt;
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : s) num_threads(nt) schedule(static)
#endif
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

static double pnorm2_masked(int n, const double* a, const uint8_t* skip, int nt) {
  double s = 0.0;
  (void)nt;
  if (!skip) return pdot(n, a, a, nt);
#ifdef _OPENMP
#pragma omp parallel for reduction(+ : s) num_threads(nt) schedule(static)
#endif
  for (int i = 0; i < n; ++i) s += skip[i] ? 0.0 : a[i] * a[i];
  return s;
}

static void pspmv(int n, const int32_t* row_ptr, const int32_t* cols, const double* values, const double* x,
                  double* y, int nt) {
  (void)nt;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) s += values[k] * x[cols[k]];
    y[i] = s;
  }
}

int afo_pcg_jacobi(int n, const int32_t* row_ptr, const int32_t* cols, const double* values, const double* b,
                   double* x, double rtol, int max_iter, const uint8_t* norm_skip, double* relres, int nb_threads) {
  int nt = nb_threads < 1 ? 1 : nb_threads;
  double* r = (double*)malloc(sizeof(double) * (size_t)n);
  double* z = (double*)malloc(sizeof(double) * (size_t)n);
  double* p = (double*)malloc(sizeof(double) * (size_t)n);
  double* q = (double*)malloc(sizeof(double) * (size_t)n);
  double* dinv = (double*)malloc(sizeof(double) * (size_t)n);
  for (int i = 0; i < n; ++i) {
    double d = 0.0;
    for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k)
      if (cols[k] == i) d = values[k];
    dinv[i] = d != 0.0 ? 1.0 / d : 1.0;
  }
  pspmv(n, row_ptr, cols, values, x, q, nt);
  for (int i = 0; i < n; ++i) r[i] = b[i] - q[i];
  double bnorm = sqrt(pnorm2_masked(n, b, norm_skip, nt));
  if (bnorm == 0.0) bnorm = 1.0;
  for (int i = 0; i < n; ++i) { z[i] = dinv[i] * r[i]; p[i] = z[i]; }
  double rz = pdot(n, r, z, nt);
  double rnorm = sqrt(pnorm2_masked(n, r, norm_skip, nt));
  int it = 0, status = 0;
  while (rnorm > rtol * bnorm && it < max_iter) {
    pspmv(n, row_ptr, cols, values, p, q, nt);
    double pq = pdot(n, p, q, nt);
    if (!(pq > 0.0)) { status = -1; break; }
    double alpha = rz / pq;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
    for (int i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      z[i] = dinv[i] * r[i];
    }
    double rz_new = pdot(n, r, z, nt);
    rnorm = sqrt(pnorm2_masked(n, r, norm_skip, nt));
    double beta = rz_new / rz;
    rz = rz_new;
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
    for (int i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  pspmv(n, row_ptr, cols, values, x, q, nt);
  double s = 0.0;
  for (int i = 0; i < n; ++i) {
    double d = b[i] - q[i];
    if (!norm_skip || !norm_skip[i]) s += d * d;
  }
  if (relres) *relres = sqrt(s) / bnorm;
  free(r); free(z); free(p); free(q); free(dinv);
  return status < 0 ? -it - 1 : it;
}
