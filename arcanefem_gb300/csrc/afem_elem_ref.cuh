// Element arithmetic in the reference's own rounding.
//
// The reference evaluates its element functions in C++ with every product and
// sum rounded on its own (its CPU build has no FMA contraction), and it forms
// the P1 tetrahedron gradients from absolute coordinates,
//   dN_0/dx = (n1.y (n3.z - n2.z) + n2.y (n1.z - n3.z) + n3.y (n2.z - n1.z)) / V6
// (femutils/ArcaneFemFunctionsGpu.h:414-535), whose terms are O(h) for a
// result of O(h^2): about log2(1 / h) bits cancel.  The Hexa8 / Quad4 Jacobians
// (femutils/ArcaneFemFunctionsGpu.h:298-350,554-586) sum absolute coordinates
// the same way.  An assembly that is merely more accurate therefore differs
// from the reference by the reference's own rounding noise: measured against
// quad-precision arithmetic at 64^3 tetrahedra, the reference formula is off
// by up to 1.65e-12 of an entry near 1e-3 of its row maximum, the cofactor
// form used by the MINIMAL kernels by 7e-14.
//
// The functions here repeat the reference's operation sequence exactly with
// __dadd_rn / __dsub_rn / __dmul_rn, which the compiler never fuses into FMAs.
// Each element row is then bit-identical to the reference's, and the gathers,
// which add the rows of a node's cells in increasing cell order starting from
// zero as the reference's node-wise loops do, make each matrix entry
// bit-identical too.  Two identities of IEEE round-to-nearest keep the count
// down without changing any value: a - b == -(b - a), and a * b == b * a, so a
// difference or product the reference forms twice (in either order) is formed
// once.  Divisions use one correctly rounded reciprocal per cell and
// Markstein's correction (below).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "afem_fp64_int.cuh"

namespace afem {
namespace ref {

__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }

// The same operations, bit for bit, on the integer pipe (afem_fp64_int.cuh),
// with the FP64 unit for the operands and results the integer path leaves out.
__device__ __forceinline__ double iadd(double a, double b) {
  uint64_t r;
  if (i64fp::add(__double_as_longlong(a), __double_as_longlong(b), &r)) return __longlong_as_double(r);
  return __dadd_rn(a, b);
}
__device__ __forceinline__ double isub(double a, double b) { return iadd(a, -b); }
__device__ __forceinline__ double imul(double a, double b) {
  uint64_t r;
  if (i64fp::mul(__double_as_longlong(a), __double_as_longlong(b), &r)) return __longlong_as_double(r);
  return __dmul_rn(a, b);
}

// Add / multiply on the FP64 pipe (INT = false) or the integer pipe (INT = true).
template <bool INT>
__device__ __forceinline__ double xadd(double a, double b) {
  if constexpr (INT) return iadd(a, b);
  else return __dadd_rn(a, b);
}
template <bool INT>
__device__ __forceinline__ double xmul(double a, double b) {
  if constexpr (INT) return imul(a, b);
  else return __dmul_rn(a, b);
}

// Biased binary exponent of x (0 for zero and subnormals, 2047 for inf / NaN).
__device__ __forceinline__ int bexp(double x) { return (__double2hiint(x) >> 20) & 0x7ff; }

// A cell measure (V6, A2, detJ) that is zero, subnormal or not finite marks a
// degenerate cell; its element matrix would be infinite or NaN.
__device__ __forceinline__ bool measure_ok(double x) {
  const int e = bexp(x);
  return e != 0 && e != 2047;
}

// Exponent window (biased 1023 +- 400) inside which the division below has no
// underflow or overflow in its quotient, remainder or correction.
__device__ __forceinline__ bool in_window(double x) {
  const int e = bexp(x);
  return e > 1023 - 400 && e < 1023 + 400;
}

// a / b rounded to nearest, given rb = RN(1 / b) (the correctly rounded
// reciprocal __drcp_rn).  q = RN(a rb) is within one ulp of a / b; the
// remainder a - b q is then exact in one FMA, and q + (a - b q) rb rounded
// once is RN(a / b): P. Markstein, "Computation of elementary functions on the
// IBM RISC System/6000 processor", IBM J. Res. Dev. 34(1), 1990 (the theorem
// on the final correction step of a division).  Three FP64 instructions
// instead of a full division per quotient.  Checked here against IEEE
// division on 3.3e9 random and edge-case operand pairs (no mismatch).  Outside
// the exponent window (and for a zero or non-finite divisor) the plain
// correctly rounded division runs instead; a zero dividend gives the signed
// zero a * rb, which is a / b.
__device__ __forceinline__ double div(double a, double b, double rb, bool b_ok) {
  if (b_ok) {
    if (in_window(a)) {
      const double q = __dmul_rn(a, rb);
      const double r = __fma_rn(-q, b, a);
      return __fma_rn(r, rb, q);
    }
    if (((__double2hiint(a) & 0x7fffffff) | __double2loint(a)) == 0) return __dmul_rn(a, rb);
  }
  return __ddiv_rn(a, b);
}

// x / D rounded to nearest for a small integer constant D: for a power of
// two the product by 1 / D is the same exact scaling; otherwise the same
// correction as above with the constant RN(1 / D).
template <int D>
__device__ __forceinline__ double div_const(double x) {
  constexpr double rd = 1.0 / D;
  if constexpr ((D & (D - 1)) == 0) {
    return __dmul_rn(x, rd);
  } else {
    if (in_window(x)) {
      const double q = __dmul_rn(x, rd);
      const double r = __fma_rn(-q, (double)D, x);
      return __fma_rn(r, rd, q);
    }
    return __ddiv_rn(x, (double)D);
  }
}

// x / 6.0 rounded to nearest (the volume of computeVolumeTetra4).
__device__ __forceinline__ double div6(double x) { return div_const<6>(x); }

// V6 = |v0 . (v1 x v2)| with v_k = n_{k+1} - n_0 (computeVolumeTetra4,
// femutils/ArcaneFemFunctionsGpu.h:113-128; math::cross / math::dot in their
// component order).
__device__ __forceinline__ double tet_v6(const double v0[3], const double v1[3], const double v2[3]) {
  const double cx = sub(mul(v1[1], v2[2]), mul(v1[2], v2[1]));
  const double cy = sub(mul(v1[2], v2[0]), mul(v1[0], v2[2]));
  const double cz = sub(mul(v1[0], v2[1]), mul(v1[1], v2[0]));
  return fabs(add(add(mul(v0[0], cx), mul(v0[1], cy)), mul(v0[2], cz)));
}

// One gradient component of the four P1 shape functions, before the division
// by V6: with a the coordinate multiplied and b the one differenced
// ((a, b) = (y, z) for d/dx, (z, x) for d/dy, (x, y) for d/dz),
//   g0 = n1.a (n3.b - n2.b) + n2.a (n1.b - n3.b) + n3.a (n2.b - n1.b)
//   g1 = n0.a (n2.b - n3.b) + n2.a (n3.b - n0.b) + n3.a (n0.b - n2.b)
//   g2 = n0.a (n3.b - n1.b) + n1.a (n0.b - n3.b) + n3.a (n1.b - n0.b)
//   g3 = n0.a (n1.b - n2.b) + n1.a (n2.b - n0.b) + n2.a (n0.b - n1.b)
// (computeGradient{X,Y,Z}Tetra4).  e[] holds the six differences
// e10 e20 e30 e21 e31 e32 (e_ij = n_i.b - n_j.b); the reverse ones are their
// negatives exactly.
template <bool INT = false>
__device__ __forceinline__ void tet_grad_numerators(const double na[4], const double e[6], double g[4]) {
  const double e10 = e[0], e20 = e[1], e30 = e[2], e21 = e[3], e31 = e[4], e32 = e[5];
  auto A = [](double x, double y) { return xadd<INT>(x, y); };
  auto M = [](double x, double y) { return xmul<INT>(x, y); };
  g[0] = A(A(M(na[1], e32), M(na[2], -e31)), M(na[3], e21));
  g[1] = A(A(M(na[0], -e32), M(na[2], e30)), M(na[3], -e20));
  g[2] = A(A(M(na[0], e31), M(na[1], -e30)), M(na[3], e10));
  g[3] = A(A(M(na[0], -e21), M(na[1], e20)), M(na[2], -e10));
}

// The reference's P1 tetrahedron geometry: gradients g[d][i] = dN_i/dx_d and
// the volume V6 / 6.  Returns V6 (zero or non-finite for a degenerate cell).
template <bool INT_DIFF = false, bool INT_NUM = false>
__device__ __forceinline__ double tet_gradients(const double n[4][3], double g[3][4], double* vol) {
  double e[3][6];
  auto D = [](double x, double y) { return xadd<INT_DIFF>(x, -y); };
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    e[k][0] = D(n[1][k], n[0][k]);
    e[k][1] = D(n[2][k], n[0][k]);
    e[k][2] = D(n[3][k], n[0][k]);
    e[k][3] = D(n[2][k], n[1][k]);
    e[k][4] = D(n[3][k], n[1][k]);
    e[k][5] = D(n[3][k], n[2][k]);
  }
  const double v0[3] = {e[0][0], e[1][0], e[2][0]};
  const double v1[3] = {e[0][1], e[1][1], e[2][1]};
  const double v2[3] = {e[0][2], e[1][2], e[2][2]};
  const double v6 = tet_v6(v0, v1, v2);
  *vol = div6(v6);
  const double rv6 = __drcp_rn(v6);
  const bool ok = in_window(v6);
  // (a, b) = (y, z), (z, x), (x, y)
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int a = (d + 1) % 3, b = (d + 2) % 3;
    const double na[4] = {n[0][a], n[1][a], n[2][a], n[3][a]};
    double num[4];
    tet_grad_numerators<INT_NUM>(na, e[b], num);
#pragma unroll
    for (int i = 0; i < 4; ++i) g[d][i] = div(num[i], v6, rv6, ok);
  }
  return v6;
}

// computeVolumeTetra4 (ArcaneFemFunctionsGpu.h:113-128): V6 / 6.
__device__ __forceinline__ double tet_volume(const double n[4][3]) {
  double v0[3], v1[3], v2[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    v0[k] = sub(n[1][k], n[0][k]);
    v1[k] = sub(n[2][k], n[0][k]);
    v2[k] = sub(n[3][k], n[0][k]);
  }
  return div6(tet_v6(v0, v1, v2));
}

// Row i of the Poisson P1 tetrahedron (_computeElementVectorTetra4Gpu,
// modules/poisson/ElementMatrix.h:107-118):
//   out_k = (vol dx_i) dx_k + (vol dy_i) dy_k + (vol dz_i) dz_k.
template <bool INT = false>
__device__ __forceinline__ void tet_row(const double g[3][4], double vol, int i, double out[4]) {
  auto A = [](double x, double y) { return xadd<INT>(x, y); };
  auto M = [](double x, double y) { return xmul<INT>(x, y); };
  const double sx = M(vol, g[0][i]), sy = M(vol, g[1][i]), sz = M(vol, g[2][i]);
#pragma unroll
  for (int k = 0; k < 4; ++k) out[k] = A(A(M(sx, g[0][k]), M(sy, g[1][k])), M(sz, g[2][k]));
}

// Triangle: area |(n1 - n0) x (n2 - n0)| / 2 (computeAreaTria3, the Real3
// cross product and normL2, ArcaneFemFunctionsGpu.h:76-86) and the gradients
// (y1 - y2, y2 - y0, y0 - y1) / A2, (x2 - x1, x0 - x2, x1 - x0) / A2 with the
// signed A2 = (x1 - x0)(y2 - y0) - (x2 - x0)(y1 - y0) (computeGradientXTria3 /
// computeGradientYTria3, :241-281).  Returns A2.
__device__ __forceinline__ double tri_gradients(const double n[3][3], double dx[3], double dy[3], double* area) {
  const double a0 = sub(n[1][0], n[0][0]), a1 = sub(n[1][1], n[0][1]), a2 = sub(n[1][2], n[0][2]);
  const double b0 = sub(n[2][0], n[0][0]), b1 = sub(n[2][1], n[0][1]), b2 = sub(n[2][2], n[0][2]);
  const double vx = sub(mul(a1, b2), mul(a2, b1));
  const double vy = sub(mul(a2, b0), mul(a0, b2));
  const double vz = sub(mul(a0, b1), mul(a1, b0));
  *area = mul(__dsqrt_rn(add(add(mul(vx, vx), mul(vy, vy)), mul(vz, vz))), 0.5);   // x / 2 == x * 0.5 exactly
  const double A2 = sub(mul(a0, b1), mul(b0, a1));
  const double rA2 = __drcp_rn(A2);
  const bool ok = in_window(A2);
  dx[0] = div(sub(n[1][1], n[2][1]), A2, rA2, ok);
  dx[1] = div(sub(n[2][1], n[0][1]), A2, rA2, ok);
  dx[2] = div(sub(n[0][1], n[1][1]), A2, rA2, ok);
  dy[0] = div(sub(n[2][0], n[1][0]), A2, rA2, ok);
  dy[1] = div(sub(n[0][0], n[2][0]), A2, rA2, ok);
  dy[2] = div(sub(n[1][0], n[0][0]), A2, rA2, ok);
  return A2;
}

// computeAreaTria3 (ArcaneFemFunctionsGpu.h:76-86): |(n1 - n0) x (n2 - n0)| / 2.
__device__ __forceinline__ double tri_area(const double n[3][3]) {
  const double a0 = sub(n[1][0], n[0][0]), a1 = sub(n[1][1], n[0][1]), a2 = sub(n[1][2], n[0][2]);
  const double b0 = sub(n[2][0], n[0][0]), b1 = sub(n[2][1], n[0][1]), b2 = sub(n[2][2], n[0][2]);
  const double vx = sub(mul(a1, b2), mul(a2, b1));
  const double vy = sub(mul(a2, b0), mul(a0, b2));
  const double vz = sub(mul(a0, b1), mul(a1, b0));
  return mul(__dsqrt_rn(add(add(mul(vx, vx), mul(vy, vy)), mul(vz, vz))), 0.5);
}

// Row i of the Poisson P1 triangle (_computeElementVectorTria3Gpu,
// modules/poisson/ElementMatrix.h:54-63): out_k = (area dx_i) dx_k + (area dy_i) dy_k.
__device__ __forceinline__ void tri_row(const double dx[3], const double dy[3], double area, int i, double out[3]) {
  const double sx = mul(area, dx[i]), sy = mul(area, dy[i]);
#pragma unroll
  for (int k = 0; k < 3; ++k) out[k] = add(mul(sx, dx[k]), mul(sy, dy[k]));
}

// Testlab B-matrix tetrahedron (_computeCellMatrixGpuTETRA4,
// modules/testlab/FemModule.h:498-538, and the row loop of
// NodeWiseCsrBiliAssembly.cc:269-290): d_k = cross products of edge
// differences, B = d / (6 vol), row i: (B_i . B_k) vol.  K[i][k] for i <= k
// (the products commute, so the matrix is symmetric bit for bit).  Returns V6.
__device__ __forceinline__ double testlab_tet(const double m[4][3], double K[4][4]) {
  auto dif = [&](int i, int j, double out[3]) {
    out[0] = sub(m[i][0], m[j][0]);
    out[1] = sub(m[i][1], m[j][1]);
    out[2] = sub(m[i][2], m[j][2]);
  };
  auto crs = [&](const double a[3], const double b[3], double out[3]) {
    out[0] = sub(mul(a[1], b[2]), mul(a[2], b[1]));
    out[1] = sub(mul(a[2], b[0]), mul(a[0], b[2]));
    out[2] = sub(mul(a[0], b[1]), mul(a[1], b[0]));
  };
  double v0[3], v1[3], v2[3];
  dif(1, 0, v0);
  dif(2, 0, v1);
  dif(3, 0, v2);
  const double v6 = tet_v6(v0, v1, v2);
  const double volume = div6(v6);
  // d0 = (m2 - m1) x (m1 - m3), d1 = (m3 - m0) x (m0 - m2),
  // d2 = (m1 - m0) x (m0 - m3), d3 = (m0 - m1) x (m1 - m2)
  double t[3], u[3], d[4][3];
  dif(2, 1, t); dif(1, 3, u); crs(t, u, d[0]);
  dif(3, 0, t); dif(0, 2, u); crs(t, u, d[1]);
  dif(1, 0, t); dif(0, 3, u); crs(t, u, d[2]);
  dif(0, 1, t); dif(1, 2, u); crs(t, u, d[3]);
  const double mlt = __drcp_rn(mul(6.0, volume));   // 1.0 / (6.0 * volume), correctly rounded
  double b[4][3];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 3; ++j) b[k][j] = mul(d[k][j], mlt);
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int k = i; k < 4; ++k)
      K[i][k] = mul(add(add(mul(b[i][0], b[k][0]), mul(b[i][1], b[k][1])), mul(b[i][2], b[k][2])), volume);
  return v6;
}

// Testlab B-matrix triangle (_computeCellMatrixGpuTRIA3, modules/testlab/FemModule.h:469-495,
// NodeWiseCsrBiliAssembly.cc:194-211), signed area: K[i][k] for i <= k.
// Returns the signed area.
__device__ __forceinline__ double testlab_tri(const double m[3][3], double K[3][3]) {
  const double area = mul(0.5, sub(mul(sub(m[1][0], m[0][0]), sub(m[2][1], m[0][1])),
                                   mul(sub(m[2][0], m[0][0]), sub(m[1][1], m[0][1]))));
  const double p[3][2] = {{sub(m[1][1], m[2][1]), sub(m[2][0], m[1][0])},
                          {sub(m[2][1], m[0][1]), sub(m[0][0], m[2][0])},
                          {sub(m[0][1], m[1][1]), sub(m[1][0], m[0][0])}};
  const double mlt = mul(0.5, __drcp_rn(area));   // 0.5 / area: exact scaling of the rounded reciprocal
  double b[3][2];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    b[k][0] = mul(p[k][0], mlt);
    b[k][1] = mul(p[k][1], mlt);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = i; k < 3; ++k) K[i][k] = mul(add(mul(b[i][0], b[k][0]), mul(b[i][1], b[k][1])), area);
  return area;
}

// ---------------------------------------------------------------------------
// Quad4 / Hexa8, 2 x 2 (x 2) Gauss points (_computeElementVectorQuad4Gpu /
// _computeElementVectorHexa8Gpu, modules/poisson/ElementMatrixHexQuad.h:63-91,
// 239-266, with computeReferenceGradients{Quad4,Hexa8},
// femutils/ShapeFunctions.h:123-129,314-345, and the Jacobians of
// femutils/ArcaneFemFunctionsGpu.h:298-350,554-586).  The Gauss-point loops
// run xi outermost, zeta innermost, at -1/sqrt3 then +1/sqrt3.

constexpr double kGaussPt = 0.57735026918962576451;

// Reference derivatives of the shape functions at Gauss point g, as the
// reference's expressions round: -0.125 * (1.0 - eta) * (1.0 - zeta) is
// (-0.125 (1 - eta)) (1 - zeta), an exact scaling followed by one rounded
// product.  Built at compile time with the same expressions.
struct HexDN {
  double v[8][3][8];   // [gauss point][d/dxi, d/deta, d/dzeta][node]
  double N[8][8];      // [gauss point][node]: 0.125 (1 -+ xi)(1 -+ eta)(1 -+ zeta)
};
constexpr HexDN make_hex_dn() {
  HexDN t{};
  for (int g = 0; g < 8; ++g) {
    const double xi = (g >> 2) ? kGaussPt : -kGaussPt, eta = ((g >> 1) & 1) ? kGaussPt : -kGaussPt,
                 zeta = (g & 1) ? kGaussPt : -kGaussPt;
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
    // shape functions as applyConstantSourceToRhsHexa8 rounds them: ((0.125 mx) me) mz
    const double mx = 1.0 - xi, px = 1.0 + xi, me = 1.0 - eta, pe = 1.0 + eta, mz = 1.0 - zeta, pz = 1.0 + zeta;
    const double Nh[8] = {0.125 * mx * me * mz, 0.125 * px * me * mz, 0.125 * px * pe * mz, 0.125 * mx * pe * mz,
                          0.125 * mx * me * pz, 0.125 * px * me * pz, 0.125 * px * pe * pz, 0.125 * mx * pe * pz};
    for (int a = 0; a < 8; ++a) {
      t.v[g][0][a] = dxi[a];
      t.v[g][1][a] = deta[a];
      t.v[g][2][a] = dzeta[a];
      t.N[g][a] = Nh[a];
    }
  }
  return t;
}

struct QuadDN {
  double v[4][2][4];   // [gauss point][d/dxi, d/deta][node]
  double N[4][4];      // [gauss point][node]: 0.25 (1 -+ xi)(1 -+ eta)
};
constexpr QuadDN make_quad_dn() {
  QuadDN t{};
  for (int g = 0; g < 4; ++g) {
    const double xi = (g >> 1) ? kGaussPt : -kGaussPt, eta = (g & 1) ? kGaussPt : -kGaussPt;
    const double dxi[4] = {-0.25 * (1.0 - eta), 0.25 * (1.0 - eta), 0.25 * (1.0 + eta), -0.25 * (1.0 + eta)};
    const double deta[4] = {-0.25 * (1.0 - xi), -0.25 * (1.0 + xi), 0.25 * (1.0 + xi), 0.25 * (1.0 - xi)};
    const double Nq[4] = {0.25 * (1.0 - xi) * (1.0 - eta), 0.25 * (1.0 + xi) * (1.0 - eta),
                          0.25 * (1.0 + xi) * (1.0 + eta), 0.25 * (1.0 - xi) * (1.0 + eta)};
    for (int a = 0; a < 4; ++a) {
      t.v[g][0][a] = dxi[a];
      t.v[g][1][a] = deta[a];
      t.N[g][a] = Nq[a];
    }
  }
  return t;
}

// Quad4 Jacobian at Gauss point g (sums of dN_a * coordinate from zero, in
// node order) and its determinant J00 J11 - J01 J10.
__device__ __forceinline__ double quad4_jacobian(const double x[4], const double y[4], const QuadDN& dn, int g,
                                                 double J[2][2]) {
  const double* dxi = dn.v[g][0];
  const double* deta = dn.v[g][1];
  double j00 = 0.0, j01 = 0.0, j10 = 0.0, j11 = 0.0;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    j00 = add(j00, mul(dxi[a], x[a]));
    j01 = add(j01, mul(dxi[a], y[a]));
    j10 = add(j10, mul(deta[a], x[a]));
    j11 = add(j11, mul(deta[a], y[a]));
  }
  J[0][0] = j00; J[0][1] = j01; J[1][0] = j10; J[1][1] = j11;
  return sub(mul(j00, j11), mul(j01, j10));
}

// Quad4 element matrix K[i][k], i <= k: sum over the Gauss points of
// ((dx_i dx_k) w + (dy_i dy_k) w), w = detJ; the Jacobian sums
// dN_a * coordinate from zero in node order; inverse = adjugate / detJ.
// Returns false if a Gauss point has a degenerate Jacobian (measure_ok).
__device__ __forceinline__ bool quad4_matrix(const double x[4], const double y[4], const QuadDN& dn, double K[4][4]) {
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int k = 0; k < 4; ++k) K[i][k] = 0.0;
  bool all_ok = true;
#pragma unroll 1
  for (int g = 0; g < 4; ++g) {
    const double* dxi = dn.v[g][0];
    const double* deta = dn.v[g][1];
    double J[2][2];
    const double det = quad4_jacobian(x, y, dn, g, J);
    const double j00 = J[0][0], j01 = J[0][1], j10 = J[1][0], j11 = J[1][1];
    all_ok &= measure_ok(det);
    const double rd = __drcp_rn(det);
    const bool ok = in_window(det);
    const double i00 = div(j11, det, rd, ok), i01 = div(-j01, det, rd, ok);
    const double i10 = div(-j10, det, rd, ok), i11 = div(j00, det, rd, ok);
    double dx[4], dy[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      dx[a] = add(mul(i00, dxi[a]), mul(i01, deta[a]));
      dy[a] = add(mul(i10, dxi[a]), mul(i11, deta[a]));
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int k = i; k < 4; ++k) K[i][k] = add(K[i][k], add(mul(mul(dx[i], dx[k]), det), mul(mul(dy[i], dy[k]), det)));
  }
  return all_ok;
}

// Hexa8 Jacobian at Gauss point g (rows d/dxi, d/deta, d/dzeta; sums of dN_a *
// coordinate from zero, in node order) and the determinant by the first row,
// J00 (J11 J22 - J12 J21) - J01 (J10 J22 - J12 J20) + J02 (J10 J21 - J11 J20);
// m[] returns those three minors.
template <bool INT = false>
__device__ __forceinline__ double hexa8_jacobian(const double x[8], const double y[8], const double z[8],
                                                 const HexDN& dn, int g, double J[3][3], double m[3]) {
  auto A = [](double p, double q) { return xadd<INT>(p, q); };
  auto M = [](double p, double q) { return xmul<INT>(p, q); };
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const double* d = dn.v[g][r];
    double s0 = 0.0, s1 = 0.0, s2 = 0.0;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      s0 = A(s0, M(d[a], x[a]));
      s1 = A(s1, M(d[a], y[a]));
      s2 = A(s2, M(d[a], z[a]));
    }
    J[r][0] = s0;
    J[r][1] = s1;
    J[r][2] = s2;
  }
  m[0] = sub(mul(J[1][1], J[2][2]), mul(J[1][2], J[2][1]));
  m[1] = sub(mul(J[1][0], J[2][2]), mul(J[1][2], J[2][0]));
  m[2] = sub(mul(J[1][0], J[2][1]), mul(J[1][1], J[2][0]));
  return add(sub(mul(J[0][0], m[0]), mul(J[0][1], m[1])), mul(J[0][2], m[2]));
}

// Hexa8 element matrix K[i][k], i <= k: sum over the Gauss points of
// (dx_i dx_k + dy_i dy_k + dz_i dz_k) detJ.  detJ by the first row,
// inverse = adjugate / detJ (the oracle's restatement of Arcane's
// math::matrixDeterminant / inverseMatrix); adjugate entries that the
// determinant already formed are its minors, negated where the reference
// writes the difference the other way round.  Returns false if a Gauss point
// has a degenerate Jacobian (measure_ok).
template <bool INT_J = false, bool INT_ROWS = false>
__device__ __forceinline__ bool hexa8_matrix(const double x[8], const double y[8], const double z[8], const HexDN& dn,
                                             double K[8][8]) {
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) K[i][k] = 0.0;
  bool all_ok = true;
#pragma unroll 1
  for (int g = 0; g < 8; ++g) {
    double J[3][3], mm[3];
    const double det = hexa8_jacobian<INT_J>(x, y, z, dn, g, J, mm);
    const double mA = mm[0], mB = mm[1], mC = mm[2];
    all_ok &= measure_ok(det);
    const double rd = __drcp_rn(det);
    const bool ok = in_window(det);
    const double v00 = div(mA, det, rd, ok);
    const double v01 = div(sub(mul(J[0][2], J[2][1]), mul(J[0][1], J[2][2])), det, rd, ok);
    const double v02 = div(sub(mul(J[0][1], J[1][2]), mul(J[0][2], J[1][1])), det, rd, ok);
    const double v10 = div(-mB, det, rd, ok);
    const double v11 = div(sub(mul(J[0][0], J[2][2]), mul(J[0][2], J[2][0])), det, rd, ok);
    const double v12 = div(sub(mul(J[0][2], J[1][0]), mul(J[0][0], J[1][2])), det, rd, ok);
    const double v20 = div(mC, det, rd, ok);
    const double v21 = div(sub(mul(J[0][1], J[2][0]), mul(J[0][0], J[2][1])), det, rd, ok);
    const double v22 = div(sub(mul(J[0][0], J[1][1]), mul(J[0][1], J[1][0])), det, rd, ok);
    const double* dxi = dn.v[g][0];
    const double* deta = dn.v[g][1];
    const double* dzeta = dn.v[g][2];
    double dx[8], dy[8], dz[8];
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      dx[a] = add(add(mul(v00, dxi[a]), mul(v01, deta[a])), mul(v02, dzeta[a]));
      dy[a] = add(add(mul(v10, dxi[a]), mul(v11, deta[a])), mul(v12, dzeta[a]));
      dz[a] = add(add(mul(v20, dxi[a]), mul(v21, deta[a])), mul(v22, dzeta[a]));
    }
    auto A = [](double p, double q) { return xadd<INT_ROWS>(p, q); };
    auto M = [](double p, double q) { return xmul<INT_ROWS>(p, q); };
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int k = i; k < 8; ++k) K[i][k] = A(K[i][k], M(A(A(M(dx[i], dx[k]), M(dy[i], dy[k])), M(dz[i], dz[k])), det));
  }
  return all_ok;
}

}  // namespace ref
}  // namespace afem
