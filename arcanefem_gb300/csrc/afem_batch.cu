// Batched Poisson P1 (2D) assembly and solve: many independent instances of
// uneven size, 4 right-hand sides each, in ONE persistent cooperative launch
// captured in a CUDA graph.
//
// The reference assembles and solves one system per module run
// (modules/poisson/FemModule.cc:163-196: _assembleBilinearOperator on the
// node-wise BSR path, _assembleLinearOperator, _solve through
// DoFLinearSystem).  Here a batch of such runs shares the GPU:
//
//  * the grid is partitioned into one TEAM of CTAs per instance, sized by a
//    cost model (rows x sqrt(rows)^(exponent - 2): Jacobi CG needs ~N
//    iterations on an N x N grid) so that the teams finish together; teams
//    never wait on each other;
//  * a team barrier is an arrival counter plus a generation word in global
//    memory; every wait is bounded (spin limit) and sets a batch error flag
//    when it runs out, after which all CTAs return;
//  * team reductions are written as per-CTA partials and summed by every CTA
//    in the same fixed order, so all CTAs of a team take the same decisions
//    (alpha, beta, convergence) without a broadcast, and results are
//    deterministic;
//  * phase A assembles each row (thread per row, element rows recomputed from
//    the incident cells in incidence order, exactly the arithmetic of the
//    node-wise gather), applies Dirichlet row-column elimination as
//    CsrDoFLinearSystemImpl does (femutils/CsrDoFLinearSystemImpl.cc:88-121,
//    column_index > 0 test included), and builds the lumped source
//    b_i = m_i f_k(x_i), f_k a sum of 8 Gaussian bumps;
//  * phase B solves the 4 systems together: a Jacobi-preconditioned FP32 CG
//    on the FP32 copy of A with reliable updates (every inner_rtol reduction
//    the correction goes into the FP64 solution and the residual is replaced
//    by the true r = b - A x, FP64 values and vectors, keeping the search
//    direction); the 4 right-hand sides are interleaved (float4 per node), so
//    each matrix entry is read once for all four.
#include <algorithm>
#include <cmath>
#include <vector>

#include "afem_krylov.cuh"

namespace afem {

constexpr int kBatchRhs = 4;
constexpr int kBumps = 8;
constexpr int kPartStride = 32;   // doubles of partials per CTA: 4 regions x 8

struct __align__(128) TeamBar {
  unsigned count;
  unsigned gen;
  unsigned pad[30];
};

struct BatchInst {
  int n, nnz, ncell, cta0, ncta, pad0, pad1, pad2;
  const double* xyz;
  const int32_t* cells;
  const int32_t* nc_ptr;
  const int32_t* nc_cell;
  const uint8_t* nc_local;
  const uint8_t* nc_slot;
  const int32_t* rp;
  const int32_t* cols;
  const uint8_t* bnd;
  const float* bumps;   // [4][8][4]
  double* vals;         // FP64 values (output)
  double* x;            // [n][4] (output)
  float* vals32;
  float* dinv;
  double* b;            // [n][4] (output)
  double* r64;          // [n][4]
  float4* r;
  float4* z;            // second direction buffer (p is double-buffered)
  float4* p;
  float4* q;
  float4* d;
  double* part;         // [ncta][kPartStride]
  TeamBar* bar;
  afem_batch_result* res;
};

struct BatchParams {
  double rtol, atol, inner_rtol;
  int max_inner, max_outer;
  long long spin_limit;
  int stall_cta;        // >= 0: that CTA leaves before its first barrier (failure-detection test)
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// ---------------------------------------------------------------------------
// Team barrier and reductions.

__device__ __forceinline__ bool team_sync(TeamBar* bar, int T, unsigned* gen_sh, int* err, long long limit) {
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned g = *gen_sh;
    __threadfence();
    if (atomicAdd(&bar->count, 1u) == (unsigned)T - 1u) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      atomicExch(&bar->gen, g + 1u);
    } else {
      long long spins = 0;
      while (*(volatile unsigned*)&bar->gen == g) {
        if (*(volatile int*)err) break;
        if (++spins > limit) {
          atomicCAS(err, 0, (int)AFEM_ERR_TIMEOUT);
          break;
        }
        __nanosleep(128);
      }
    }
    __threadfence();
    *gen_sh = g + 1u;
  }
  __syncthreads();
  return *(volatile int*)err == 0;
}

// Sum v[0..M) over the block and then over the team (fixed order); the
// results land in out[0..M) for every thread of every CTA of the team.
// `region` (0..3) selects the partials slot (see the phase notes below).
// T = float for the inner-solve dot products: per-thread and per-warp sums
// stay on the FP32 pipe (GB300 issues FP64 at 1/74 of FP32, and the per-row
// FP64 accumulation bound this kernel), only warp totals go to FP64.
template <int BLOCK, int M, class T>
__device__ __forceinline__ bool team_reduce(const T (&v)[M], double (&out)[M], const BatchInst& I, int rank,
                                            int region, double (*red)[8], double* tres, unsigned* gen_sh, int* err,
                                            long long limit) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < M; ++j) {
    T s = v[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) red[warp][j] = (double)s;
  }
  __syncthreads();
  if (threadIdx.x < M) {
    double s = 0.0;
    for (int w = 0; w < BLOCK / 32; ++w) s += red[w][threadIdx.x];
    I.part[(int64_t)rank * kPartStride + region * 8 + threadIdx.x] = s;
  }
  if (!team_sync(I.bar, I.ncta, gen_sh, err, limit)) return false;
  for (int j = warp; j < M; j += BLOCK / 32) {
    double s = 0.0;
    for (int k = lane; k < I.ncta; k += 32)
      s += ((volatile const double*)I.part)[(int64_t)k * kPartStride + region * 8 + j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) tres[j] = s;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < M; ++j) out[j] = tres[j];
  __syncthreads();
  return true;
}

// ---------------------------------------------------------------------------
// Phase A: one row of the Poisson operator, its elimination, the source.

__device__ __forceinline__ void assemble_row(const BatchInst& I, int row) {
  const int32_t rb = I.rp[row], re = I.rp[row + 1];
  for (int32_t k = rb; k < re; ++k) I.vals[k] = 0.0;
  const int32_t p0 = I.nc_ptr[row], p1 = I.nc_ptr[row + 1];
  double diag = 0.0, mass = 0.0;
  for (int32_t p = p0; p < p1; ++p) {
    const int32_t c = I.nc_cell[p];
    const int li = I.nc_local[p];
    const int32_t* qn = I.cells + 3 * (int64_t)c;
    const double* a0 = I.xyz + 3 * (int64_t)qn[0];
    const double* a1 = I.xyz + 3 * (int64_t)qn[1];
    const double* a2 = I.xyz + 3 * (int64_t)qn[2];
    const double x0 = a0[0], y0 = a0[1];
    const double v1x = a1[0] - x0, v1y = a1[1] - y0;
    const double v2x = a2[0] - x0, v2y = a2[1] - y0;
    const double A2 = v1x * v2y - v1y * v2x;
    const double s = 1.0 / (2.0 * fabs(A2));
    const double c0x = v1y - v2y, c0y = v2x - v1x;
    const double k01 = s * (c0x * v2y - c0y * v2x);
    const double k02 = s * (c0y * v1x - c0x * v1y);
    const double k12 = s * (-(v2y * v1y) - v2x * v1x);
    double e0, e1, e2;
    if (li == 0) { e0 = -(k01 + k02); e1 = k01; e2 = k02; }
    else if (li == 1) { e0 = -(k01 + k12); e1 = k01; e2 = k12; }
    else { e0 = -(k02 + k12); e1 = k02; e2 = k12; }
    const uint8_t* sp = I.nc_slot + 3 * (int64_t)p;
    diag += e0;
    I.vals[rb + sp[1]] += e1;
    I.vals[rb + sp[2]] += e2;
    mass += fabs(A2) / 6.0;
  }
  if (p1 > p0) I.vals[rb + I.nc_slot[3 * (int64_t)p0]] = diag;
  // row-column elimination (u = 0), column_index > 0 test as the reference
  const bool brow = I.bnd[row] != 0;
  double dval = 1.0;
  for (int32_t k = rb; k < re; ++k) {
    const int32_t c = I.cols[k];
    double v = I.vals[k];
    if (c > 0 && (brow || I.bnd[c])) {
      v = (c == row) ? 1.0 : 0.0;
      I.vals[k] = v;
    }
    if (c == row) dval = v;
    I.vals32[k] = (float)v;
  }
  I.dinv[row] = (float)(1.0 / (dval != 0.0 ? dval : 1.0));
  // lumped source and zero initial guess; b = 0 on eliminated rows
  const float px = (float)I.xyz[3 * (int64_t)row], py = (float)I.xyz[3 * (int64_t)row + 1];
#pragma unroll
  for (int j = 0; j < kBatchRhs; ++j) {
    float f = 0.f;
    const float* bp = I.bumps + j * kBumps * 4;
    for (int m = 0; m < kBumps; ++m) {
      const float dx = px - bp[4 * m + 1], dy = py - bp[4 * m + 2], w = bp[4 * m + 3];
      f += bp[4 * m] * expf(-(dx * dx + dy * dy) / (2.f * w * w));
    }
    I.b[(int64_t)row * kBatchRhs + j] = brow ? 0.0 : mass * (double)f;
    I.x[(int64_t)row * kBatchRhs + j] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// The persistent kernel.

constexpr int kRowUnroll = 8;   // entries of a row loaded together in the FP32 SpMV (2D P1 rows hold ~7)

// Per-CTA copy of the team's solver scalars (identical in every CTA of a team).
struct SolveState {
  double bnorm2[kBatchRhs], tol2[kBatchRhs], rr64[kBatchRhs], itol2[kBatchRhs], rz[kBatchRhs], rzprev[kBatchRhs];
  float alpha[kBatchRhs], beta[kBatchRhs], zc[kBatchRhs];
  int active[kBatchRhs], keep[kBatchRhs];
  int any, all_done;
};

template <int BLOCK>
__global__ void __launch_bounds__(BLOCK, 1024 / BLOCK) k_batch(const BatchInst* __restrict__ insts,
                                                               const int32_t* __restrict__ cta_team, BatchParams prm,
                                                               int* err) {
  __shared__ BatchInst I;
  __shared__ SolveState S;
  __shared__ double red[BLOCK / 32][8];
  __shared__ double tres[8];
  __shared__ unsigned gen_sh;
  const int team = cta_team[blockIdx.x];
  if (threadIdx.x == 0) {
    I = insts[team];
    gen_sh = 0u;
  }
  __syncthreads();
  const int rank = blockIdx.x - I.cta0;
  const int nthr = I.ncta * BLOCK;
  const int tid = rank * BLOCK + threadIdx.x;
  const long long lim = prm.spin_limit;
  const unsigned long long t_start = globaltimer_ns();
  if ((int)blockIdx.x == prm.stall_cta) return;   // failure-detection test: this CTA never arrives

  // ---- phase A: assembly
  for (int row = tid; row < I.n; row += nthr) assemble_row(I, row);
  if (!team_sync(I.bar, I.ncta, &gen_sh, err, lim)) return;

  // ---- phase B: FP64 refinement around FP32 Jacobi CG, 4 right-hand sides
  // Partials regions: 0 = <p,q>, 1 = <r,z>,<r,r> (inner), 2 = outer residual
  // norms, 3 = initial <r,z> of an inner solve.  Consecutive uses of one
  // region are always separated by at least two team barriers.
  int inner_total = 0, outer = 0, status = AFEM_OK;
  for (;; ++outer) {
    {
      double loc[2 * kBatchRhs] = {};
      for (int row = tid; row < I.n; row += nthr) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        for (int32_t k = I.rp[row]; k < I.rp[row + 1]; ++k) {
          const double a = I.vals[k];
          const double2* xc = reinterpret_cast<const double2*>(I.x + (int64_t)I.cols[k] * kBatchRhs);
          const double2 u = xc[0], w = xc[1];
          s0 += a * u.x; s1 += a * u.y; s2 += a * w.x; s3 += a * w.y;
        }
        const double* br = I.b + (int64_t)row * kBatchRhs;
        double* rr = I.r64 + (int64_t)row * kBatchRhs;
        const double r0 = br[0] - s0, r1 = br[1] - s1, r2 = br[2] - s2, r3 = br[3] - s3;
        rr[0] = r0; rr[1] = r1; rr[2] = r2; rr[3] = r3;
        loc[0] += r0 * r0; loc[1] += r1 * r1; loc[2] += r2 * r2; loc[3] += r3 * r3;
        loc[4] += br[0] * br[0]; loc[5] += br[1] * br[1]; loc[6] += br[2] * br[2]; loc[7] += br[3] * br[3];
      }
      double tot[2 * kBatchRhs];
      if (!team_reduce<BLOCK, 2 * kBatchRhs>(loc, tot, I, rank, 2, red, tres, &gen_sh, err, lim)) return;
      if (threadIdx.x == 0) {
        int all = 1;
        for (int j = 0; j < kBatchRhs; ++j) {
          if (outer == 0) {
            S.bnorm2[j] = tot[kBatchRhs + j];
            S.tol2[j] = fmax(prm.rtol * prm.rtol * S.bnorm2[j], prm.atol * prm.atol);
          }
          // keep the direction when the last cycle at least halved the true
          // residual and cycles are short enough for the FP32 recursive
          // residual to stay close to the true one (inner_rtol >= 0.01)
          S.keep[j] = outer > 0 && prm.inner_rtol >= 0.01 && tot[j] <= 0.25 * S.rr64[j];
          S.rr64[j] = tot[j];
          const int dn = !(tot[j] > S.tol2[j]);
          S.active[j] = !dn;
          S.itol2[j] = prm.inner_rtol * prm.inner_rtol * tot[j];
          all = all && dn;
        }
        S.all_done = all;
      }
      __syncthreads();
    }
    if (S.all_done) break;
    if (outer >= prm.max_outer) {
      status = AFEM_ERR_NOT_CONVERGED;
      break;
    }
    // FP32 CG on A32 d = r32 from d = 0 for the unconverged right-hand sides.
    // z = D^-1 r is never stored: the SpMV of each iteration forms the new
    // direction p = zc D^-1 r + beta p_old of every entry it gathers (and
    // writes its own row), so the direction update needs no pass and no
    // barrier of its own; p is double-buffered (p_old is read while p is
    // written), with the parity of the running iteration count so that a
    // direction survives from one cycle to the next.  A right-hand side that
    // has reached its cycle tolerance keeps its direction (zc = 0, beta = 1).
    // Reliable updates: the cycle's residual is the true FP64 one, and the
    // direction is kept (beta = <r,z>_new / <r,z>_prev) unless the last cycle
    // failed to halve the true residual.
    {
      float lrz[kBatchRhs] = {};
      const bool a0 = S.active[0], a1 = S.active[1], a2 = S.active[2], a3 = S.active[3];
      for (int row = tid; row < I.n; row += nthr) {
        const double* rr = I.r64 + (int64_t)row * kBatchRhs;
        const float di = I.dinv[row];
        const float4 rv = make_float4(a0 ? (float)rr[0] : 0.f, a1 ? (float)rr[1] : 0.f, a2 ? (float)rr[2] : 0.f,
                                      a3 ? (float)rr[3] : 0.f);
        I.r[row] = rv;
        if (outer == 0) I.z[row] = make_float4(0.f, 0.f, 0.f, 0.f);   // p_old of the first iteration
        I.d[row] = make_float4(0.f, 0.f, 0.f, 0.f);
        lrz[0] = fmaf(rv.x, di * rv.x, lrz[0]); lrz[1] = fmaf(rv.y, di * rv.y, lrz[1]);
        lrz[2] = fmaf(rv.z, di * rv.z, lrz[2]); lrz[3] = fmaf(rv.w, di * rv.w, lrz[3]);
      }
      double trz[kBatchRhs];
      if (!team_reduce<BLOCK, kBatchRhs>(lrz, trz, I, rank, 3, red, tres, &gen_sh, err, lim)) return;
      if (threadIdx.x == 0)
        for (int j = 0; j < kBatchRhs; ++j) {
          S.beta[j] = S.keep[j] && S.active[j] ? (float)(trz[j] / S.rzprev[j]) : 0.f;
          S.zc[j] = 1.f;
          S.rz[j] = trz[j];
        }
      __syncthreads();
    }
    for (int it = 0; it < prm.max_inner; ++it) {
      float4* const pold = (inner_total & 1) ? I.p : I.z;
      float4* const pnew = (inner_total & 1) ? I.z : I.p;
      // p = D^-1 r + beta p_old (on the fly), q = A32 p ; <p, q>.  Thread per
      // row; the row's column and value loads are issued together, then its gathers.
      {
        const float b0 = S.beta[0], b1 = S.beta[1], b2 = S.beta[2], b3 = S.beta[3];
        const float z0 = S.zc[0], z1 = S.zc[1], z2 = S.zc[2], z3 = S.zc[3];
        float lpq[kBatchRhs] = {};
        for (int row = tid; row < I.n; row += nthr) {
          const int32_t rb = I.rp[row], e = I.rp[row + 1];
          const int len = e - rb;
          int32_t c[kRowUnroll];
          float a[kRowUnroll];
#pragma unroll
          for (int u = 0; u < kRowUnroll; ++u) {
            c[u] = u < len ? I.cols[rb + u] : row;
            a[u] = u < len ? I.vals32[rb + u] : 0.f;
          }
          float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
          for (int u = 0; u < kRowUnroll; ++u) {
            const float4 rv = I.r[c[u]], po = pold[c[u]];
            const float di = I.dinv[c[u]];
            const float4 pv = make_float4(fmaf(b0, po.x, z0 * di * rv.x), fmaf(b1, po.y, z1 * di * rv.y),
                                          fmaf(b2, po.z, z2 * di * rv.z), fmaf(b3, po.w, z3 * di * rv.w));
            s.x = fmaf(a[u], pv.x, s.x); s.y = fmaf(a[u], pv.y, s.y);
            s.z = fmaf(a[u], pv.z, s.z); s.w = fmaf(a[u], pv.w, s.w);
          }
          for (int32_t k = rb + kRowUnroll; k < e; ++k) {
            const int32_t ck = I.cols[k];
            const float av = I.vals32[k];
            const float4 rv = I.r[ck], po = pold[ck];
            const float di = I.dinv[ck];
            const float4 pv = make_float4(fmaf(b0, po.x, z0 * di * rv.x), fmaf(b1, po.y, z1 * di * rv.y),
                                          fmaf(b2, po.z, z2 * di * rv.z), fmaf(b3, po.w, z3 * di * rv.w));
            s.x = fmaf(av, pv.x, s.x); s.y = fmaf(av, pv.y, s.y); s.z = fmaf(av, pv.z, s.z); s.w = fmaf(av, pv.w, s.w);
          }
          const float4 rv = I.r[row], po = pold[row];
          const float di = I.dinv[row];
          const float4 pr = make_float4(fmaf(b0, po.x, z0 * di * rv.x), fmaf(b1, po.y, z1 * di * rv.y),
                                        fmaf(b2, po.z, z2 * di * rv.z), fmaf(b3, po.w, z3 * di * rv.w));
          pnew[row] = pr;
          I.q[row] = s;
          lpq[0] = fmaf(pr.x, s.x, lpq[0]); lpq[1] = fmaf(pr.y, s.y, lpq[1]);
          lpq[2] = fmaf(pr.z, s.z, lpq[2]); lpq[3] = fmaf(pr.w, s.w, lpq[3]);
        }
        double pq[kBatchRhs];
        if (!team_reduce<BLOCK, kBatchRhs>(lpq, pq, I, rank, 0, red, tres, &gen_sh, err, lim)) return;
        if (threadIdx.x == 0) {
          for (int j = 0; j < kBatchRhs; ++j) {
            if (S.active[j] && !(pq[j] > 0.0)) {   // breakdown: stop this right-hand side
              S.active[j] = 0;
              status = AFEM_ERR_BREAKDOWN;
            }
            S.alpha[j] = S.active[j] ? (float)(S.rz[j] / pq[j]) : 0.f;
          }
        }
        __syncthreads();
      }
      // d += alpha p ; r -= alpha q ; <r, D^-1 r>, <r, r>
      {
        const float al0 = S.alpha[0], al1 = S.alpha[1], al2 = S.alpha[2], al3 = S.alpha[3];
        float lrr[2 * kBatchRhs] = {};
        for (int row = tid; row < I.n; row += nthr) {
          const float4 pv = pnew[row], qv = I.q[row];
          float4 dv = I.d[row], rv = I.r[row];
          dv.x = fmaf(al0, pv.x, dv.x); dv.y = fmaf(al1, pv.y, dv.y);
          dv.z = fmaf(al2, pv.z, dv.z); dv.w = fmaf(al3, pv.w, dv.w);
          rv.x = fmaf(-al0, qv.x, rv.x); rv.y = fmaf(-al1, qv.y, rv.y);
          rv.z = fmaf(-al2, qv.z, rv.z); rv.w = fmaf(-al3, qv.w, rv.w);
          const float di = I.dinv[row];
          I.d[row] = dv;
          I.r[row] = rv;
          lrr[0] = fmaf(rv.x, di * rv.x, lrr[0]); lrr[1] = fmaf(rv.y, di * rv.y, lrr[1]);
          lrr[2] = fmaf(rv.z, di * rv.z, lrr[2]); lrr[3] = fmaf(rv.w, di * rv.w, lrr[3]);
          lrr[4] = fmaf(rv.x, rv.x, lrr[4]); lrr[5] = fmaf(rv.y, rv.y, lrr[5]);
          lrr[6] = fmaf(rv.z, rv.z, lrr[6]); lrr[7] = fmaf(rv.w, rv.w, lrr[7]);
        }
        double trr[2 * kBatchRhs];
        if (!team_reduce<BLOCK, 2 * kBatchRhs>(lrr, trr, I, rank, 1, red, tres, &gen_sh, err, lim)) return;
        if (threadIdx.x == 0) {
          int any = 0;
          for (int j = 0; j < kBatchRhs; ++j) {
            if (S.active[j]) {
              S.beta[j] = (float)(trr[j] / S.rz[j]);
              S.rzprev[j] = S.rz[j];
              S.rz[j] = trr[j];
              if (!(trr[kBatchRhs + j] > S.itol2[j])) S.active[j] = 0;
            }
            if (!S.active[j]) {   // keep the direction for the next cycle
              S.beta[j] = 1.f;
              S.zc[j] = 0.f;
            }
            any = any || S.active[j];
          }
          S.any = any;
        }
        __syncthreads();
      }
      ++inner_total;
      if (!S.any) break;
    }
    // x += d (FP64); the next residual reads neighbours' x
    for (int row = tid; row < I.n; row += nthr) {
      const float4 dv = I.d[row];
      double* xr = I.x + (int64_t)row * kBatchRhs;
      xr[0] += (double)dv.x; xr[1] += (double)dv.y; xr[2] += (double)dv.z; xr[3] += (double)dv.w;
    }
    if (!team_sync(I.bar, I.ncta, &gen_sh, err, lim)) return;
  }
  if (rank == 0 && threadIdx.x == 0) {
    I.res->finish_ms = (float)((double)(globaltimer_ns() - t_start) * 1e-6);
    I.res->inner_iterations = inner_total;
    I.res->refinements = outer;
    I.res->status = status;
    for (int j = 0; j < kBatchRhs; ++j)
      I.res->relres[j] = S.bnorm2[j] > 0.0 ? sqrt(S.rr64[j] / S.bnorm2[j]) : sqrt(S.rr64[j]);
  }
}

}  // namespace afem

// ---------------------------------------------------------------------------
// Host side.

using namespace afem;

struct afem_batch_s {
  afem_context ctx = nullptr;
  int ninst = 0;
  std::vector<afem_batch_instance> inst;
  std::vector<BatchInst> dinst;     // host copy of the descriptors (device pointers)
  BatchInst* insts_d = nullptr;
  int32_t* cta_team_d = nullptr;
  TeamBar* bars_d = nullptr;
  afem_batch_result* res_d = nullptr;
  int* err_d = nullptr;
  double* part_d = nullptr;
  std::vector<void*> owned;
  afem_batch_config cfg{256, 4, 3.5f};
  std::vector<double> weights;      // empty: the cost model
  int grid = 0;
  int max_teams = 0;
  // graph of the current configuration and options
  GraphChunk* graph = nullptr;
  BatchParams graph_prm{};
  bool graph_valid = false;
};

namespace afem {

static afem_status batch_alloc(afem_batch b, size_t bytes, void** out) {
  AFEM_CUDA(cudaMallocAsync(out, std::max<size_t>(bytes, 16), b->ctx->stream));
  b->owned.push_back(*out);
  return AFEM_OK;
}

template <int BLOCK>
static int max_blocks_per_sm() {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<BLOCK>, BLOCK, 0);
  return nb;
}

static int occupancy(int block) {
  switch (block) {
    case 128: return max_blocks_per_sm<128>();
    case 256: return max_blocks_per_sm<256>();
    case 512: return max_blocks_per_sm<512>();
    default: return 0;
  }
}

// Team sizes: every instance gets >= 1 CTA, the rest in proportion to
// rows^(exponent / 2) (largest remainders first); deterministic.
// Explicit weights (afem_batch_set_weights) replace the cost model.
static void team_sizes(const std::vector<afem_batch_instance>& inst, const std::vector<double>& weights, int grid,
                       float exponent, std::vector<int>& out) {
  const int n = (int)inst.size();
  std::vector<double> w(n);
  double tot = 0.0;
  for (int i = 0; i < n; ++i) {
    w[i] = weights.empty() ? std::pow((double)std::max(inst[i].nb_node, 1), exponent / 2.0) : weights[i];
    tot += w[i];
  }
  out.assign(n, 1);
  const int spare = grid - n;
  std::vector<std::pair<double, int>> frac(n);
  int used = 0;
  for (int i = 0; i < n; ++i) {
    const double share = spare * w[i] / tot;
    const int whole = (int)std::floor(share);
    out[i] += whole;
    used += whole;
    frac[i] = {share - whole, i};
  }
  std::sort(frac.begin(), frac.end(), [](const std::pair<double, int>& a, const std::pair<double, int>& b) {
    return a.first != b.first ? a.first > b.first : a.second < b.second;
  });
  for (int k = 0; k < spare - used; ++k) out[frac[k % n].second] += 1;
}

static afem_status batch_configure(afem_batch b) {
  afem_context ctx = b->ctx;
  const int occ = occupancy(b->cfg.block);
  if (occ <= 0) return fail(AFEM_ERR_BAD_ARG, "afem_batch: block size %d not supported (128, 256 or 512)", b->cfg.block);
  const int bps = std::min(b->cfg.blocks_per_sm, occ);
  AFEM_CHECK_ARG(bps >= 1, "afem_batch: blocks_per_sm must be >= 1");
  const int grid = ctx->sm_count * bps;
  AFEM_CHECK_ARG(grid >= b->ninst, "afem_batch: %d instances need at least as many CTAs (grid %d)", b->ninst, grid);
  std::vector<int> sizes;
  team_sizes(b->inst, b->weights, grid, b->cfg.cost_exponent, sizes);
  std::vector<int32_t> cta_team(grid);
  int c = 0;
  for (int i = 0; i < b->ninst; ++i) {
    b->dinst[i].cta0 = c;
    b->dinst[i].ncta = sizes[i];
    for (int k = 0; k < sizes[i]; ++k) cta_team[c++] = i;
  }
  // partials: one region block per CTA, laid out by team
  for (int i = 0; i < b->ninst; ++i) b->dinst[i].part = b->part_d + (size_t)b->dinst[i].cta0 * kPartStride;
  AFEM_CUDA(cudaMemcpyAsync(b->insts_d, b->dinst.data(), sizeof(BatchInst) * b->ninst, cudaMemcpyHostToDevice,
                            ctx->stream));
  AFEM_CUDA(cudaMemcpyAsync(b->cta_team_d, cta_team.data(), sizeof(int32_t) * grid, cudaMemcpyHostToDevice,
                            ctx->stream));
  AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
  b->grid = grid;
  b->graph_valid = false;
  return AFEM_OK;
}

template <int BLOCK>
static cudaError_t launch_batch(afem_batch b, cudaStream_t s, const BatchParams& prm) {
  cudaLaunchConfig_t lc = {};
  lc.gridDim = dim3(b->grid);
  lc.blockDim = dim3(BLOCK);
  lc.dynamicSmemBytes = 0;
  lc.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  lc.attrs = attr;
  lc.numAttrs = 1;
  return cudaLaunchKernelEx(&lc, k_batch<BLOCK>, (const BatchInst*)b->insts_d, (const int32_t*)b->cta_team_d, prm,
                            b->err_d);
}

static afem_status batch_enqueue(afem_batch b, cudaStream_t s, const BatchParams& prm) {
  AFEM_CUDA(cudaMemsetAsync(b->bars_d, 0, sizeof(TeamBar) * b->ninst, s));
  AFEM_CUDA(cudaMemsetAsync(b->err_d, 0, sizeof(int), s));
  AFEM_CUDA(cudaMemsetAsync(b->res_d, 0, sizeof(afem_batch_result) * b->ninst, s));
  cudaError_t e = cudaErrorInvalidValue;
  switch (b->cfg.block) {
    case 128: e = launch_batch<128>(b, s, prm); break;
    case 256: e = launch_batch<256>(b, s, prm); break;
    case 512: e = launch_batch<512>(b, s, prm); break;
  }
  if (e != cudaSuccess) return cuda_fail(e, "k_batch cooperative launch", __FILE__, __LINE__);
  b->ctx->launches += 1;
  return AFEM_OK;
}

static BatchParams batch_params(const afem_solver_options& opt) {
  BatchParams prm{};
  prm.rtol = opt.rtol;
  prm.atol = opt.atol;
  prm.inner_rtol = opt.inner_rtol > 0 ? opt.inner_rtol : 0.1;
  prm.max_inner = opt.max_iter > 0 ? opt.max_iter : 1000;
  prm.max_outer = 30;
  prm.spin_limit = 20000000LL;   // ~2.5 s of 128 ns sleeps
  prm.stall_cta = -1;
  return prm;
}

static bool same_params(const BatchParams& a, const BatchParams& c) {
  return a.rtol == c.rtol && a.atol == c.atol && a.inner_rtol == c.inner_rtol && a.max_inner == c.max_inner &&
         a.max_outer == c.max_outer && a.spin_limit == c.spin_limit && a.stall_cta == c.stall_cta;
}

static afem_status batch_run(afem_batch b, const BatchParams& prm, bool use_graph, float* ms) {
  afem_context ctx = b->ctx;
  if (use_graph && (!b->graph_valid || !same_params(prm, b->graph_prm))) {
    delete b->graph;
    b->graph = new (std::nothrow) GraphChunk();
    if (!b->graph) return fail(AFEM_ERR_OOM, "afem_batch: host allocation");
    AFEM_TRY(capture(ctx, *b->graph, [&](cudaStream_t s) { return batch_enqueue(b, s, prm); }));
    b->graph_prm = prm;
    b->graph_valid = true;
  }
  cudaEvent_t e0, e1;
  AFEM_CUDA(cudaEventCreate(&e0));
  AFEM_CUDA(cudaEventCreate(&e1));
  AFEM_CUDA(cudaEventRecord(e0, ctx->stream));
  afem_status st = AFEM_OK;
  if (use_graph) {
    cudaError_t e = cudaGraphLaunch(b->graph->exec, ctx->stream);
    if (e != cudaSuccess) st = cuda_fail(e, "cudaGraphLaunch", __FILE__, __LINE__);
    else ctx->launches += 1;
  } else {
    st = batch_enqueue(b, ctx->stream, prm);
  }
  cudaEventRecord(e1, ctx->stream);
  cudaError_t se = cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != AFEM_OK) return st;
  if (se != cudaSuccess) return cuda_fail(se, "afem_batch_solve", __FILE__, __LINE__);
  if (ms) *ms = t;
  int err = 0;
  AFEM_TRY(read_scalar(ctx, b->err_d, &err));
  if (err) return fail((afem_status)err, "afem_batch: a team barrier wait ran out (status %d)", err);
  return AFEM_OK;
}

}  // namespace afem

extern "C" {

afem_status afem_batch_create(afem_context ctx, int nb_inst, const afem_batch_instance* inst_h, afem_batch* out) {
  AFEM_CHECK_ARG(ctx && inst_h && out && nb_inst >= 1, "afem_batch_create: bad arguments");
  *out = nullptr;
  afem_batch b = new (std::nothrow) afem_batch_s();
  if (!b) return fail(AFEM_ERR_OOM, "afem_batch_create: host allocation");
  b->ctx = ctx;
  b->ninst = nb_inst;
  b->inst.assign(inst_h, inst_h + nb_inst);
  b->dinst.resize(nb_inst);
  auto cleanup = [&](afem_status st) {
    afem_batch_destroy(b);
    return st;
  };
  afem_status st;
  for (int i = 0; i < nb_inst; ++i) {
    const afem_batch_instance& s = inst_h[i];
    if (s.nb_node <= 0 || s.nb_cell <= 0 || !s.coords_d || !s.cells_d || !s.nc_ptr_d || !s.nc_cell_d ||
        !s.nc_local_d || !s.nc_slot_d || !s.row_ptr_d || !s.cols_d || !s.dirichlet_d || !s.sources_d ||
        !s.values_d || !s.rhs_d || !s.x_d)
      return cleanup(fail(AFEM_ERR_BAD_ARG, "afem_batch_create: instance %d incomplete", i));
    if (((uintptr_t)s.x_d & 15) != 0)
      return cleanup(fail(AFEM_ERR_BAD_ARG, "afem_batch_create: instance %d x_d must be 16-byte aligned", i));
    int32_t nnz = 0;
    if ((st = read_scalar(ctx, s.row_ptr_d + s.nb_node, &nnz)) != AFEM_OK) return cleanup(st);
    BatchInst& d = b->dinst[i];
    d = BatchInst{};
    d.n = s.nb_node;
    d.nnz = nnz;
    d.ncell = s.nb_cell;
    d.xyz = s.coords_d;
    d.cells = s.cells_d;
    d.nc_ptr = s.nc_ptr_d;
    d.nc_cell = s.nc_cell_d;
    d.nc_local = s.nc_local_d;
    d.nc_slot = s.nc_slot_d;
    d.rp = s.row_ptr_d;
    d.cols = s.cols_d;
    d.bnd = s.dirichlet_d;
    d.bumps = s.sources_d;
    d.vals = s.values_d;
    d.x = s.x_d;
    const size_t n = s.nb_node;
    void* pv;
    if ((st = batch_alloc(b, sizeof(float) * (size_t)nnz, &pv))) return cleanup(st);
    d.vals32 = (float*)pv;
    if ((st = batch_alloc(b, sizeof(float) * n, &pv))) return cleanup(st);
    d.dinv = (float*)pv;
    d.b = s.rhs_d;
    if ((st = batch_alloc(b, sizeof(double) * kBatchRhs * n, &pv))) return cleanup(st);
    d.r64 = (double*)pv;
    float4** vecs[5] = {&d.r, &d.z, &d.p, &d.q, &d.d};
    for (float4** v : vecs) {
      if ((st = batch_alloc(b, sizeof(float4) * n, &pv))) return cleanup(st);
      *v = (float4*)pv;
    }
  }
  void* pv;
  const int max_grid = ctx->sm_count * 8;
  if ((st = batch_alloc(b, sizeof(BatchInst) * nb_inst, &pv))) return cleanup(st);
  b->insts_d = (BatchInst*)pv;
  if ((st = batch_alloc(b, sizeof(int32_t) * max_grid, &pv))) return cleanup(st);
  b->cta_team_d = (int32_t*)pv;
  if ((st = batch_alloc(b, sizeof(TeamBar) * nb_inst, &pv))) return cleanup(st);
  b->bars_d = (TeamBar*)pv;
  if ((st = batch_alloc(b, sizeof(afem_batch_result) * nb_inst, &pv))) return cleanup(st);
  b->res_d = (afem_batch_result*)pv;
  if ((st = batch_alloc(b, sizeof(int), &pv))) return cleanup(st);
  b->err_d = (int*)pv;
  if ((st = batch_alloc(b, sizeof(double) * kPartStride * max_grid, &pv))) return cleanup(st);
  b->part_d = (double*)pv;
  for (int i = 0; i < nb_inst; ++i) {
    b->dinst[i].bar = b->bars_d + i;
    b->dinst[i].res = b->res_d + i;
  }
  if ((st = batch_configure(b)) != AFEM_OK) return cleanup(st);
  *out = b;
  return AFEM_OK;
}

afem_status afem_batch_destroy(afem_batch b) {
  if (!b) return AFEM_OK;
  delete b->graph;
  for (void* p : b->owned) cudaFreeAsync(p, b->ctx->stream);
  cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return AFEM_OK;
}

afem_status afem_batch_set_config(afem_batch b, const afem_batch_config* cfg) {
  AFEM_CHECK_ARG(b && cfg, "afem_batch_set_config: null argument");
  AFEM_CHECK_ARG(cfg->block == 128 || cfg->block == 256 || cfg->block == 512,
                 "afem_batch_set_config: block must be 128, 256 or 512");
  AFEM_CHECK_ARG(cfg->blocks_per_sm >= 1 && cfg->blocks_per_sm <= 8, "afem_batch_set_config: blocks_per_sm 1..8");
  AFEM_CHECK_ARG(cfg->cost_exponent >= 0.f && cfg->cost_exponent <= 6.f, "afem_batch_set_config: cost_exponent 0..6");
  const afem_batch_config old = b->cfg;
  b->cfg = *cfg;
  afem_status st = batch_configure(b);
  if (st != AFEM_OK) {
    b->cfg = old;
    batch_configure(b);
  }
  return st;
}

afem_status afem_batch_get_config(afem_batch b, afem_batch_config* cfg, int* grid) {
  AFEM_CHECK_ARG(b && cfg, "afem_batch_get_config: null argument");
  *cfg = b->cfg;
  if (grid) *grid = b->grid;
  return AFEM_OK;
}

afem_status afem_batch_set_weights(afem_batch b, const double* weights_h) {
  AFEM_CHECK_ARG(b, "afem_batch_set_weights: null batch");
  std::vector<double> old = b->weights;
  if (weights_h) {
    b->weights.assign(weights_h, weights_h + b->ninst);
    for (double w : b->weights)
      if (!(w > 0.0) || !std::isfinite(w)) {
        b->weights = old;
        return fail(AFEM_ERR_BAD_ARG, "afem_batch_set_weights: weights must be positive and finite");
      }
  } else {
    b->weights.clear();
  }
  afem_status st = batch_configure(b);
  if (st != AFEM_OK) {
    b->weights = old;
    batch_configure(b);
  }
  return st;
}

afem_status afem_batch_team(afem_batch b, int inst, int* cta0, int* ncta) {
  AFEM_CHECK_ARG(b && inst >= 0 && inst < b->ninst && cta0 && ncta, "afem_batch_team: bad arguments");
  *cta0 = b->dinst[inst].cta0;
  *ncta = b->dinst[inst].ncta;
  return AFEM_OK;
}

afem_status afem_batch_solve(afem_batch b, const afem_solver_options* opt_in, afem_batch_result* results_h,
                             float* ms) {
  AFEM_CHECK_ARG(b, "afem_batch_solve: null batch");
  afem_solver_options opt;
  if (opt_in) opt = *opt_in;
  else afem_solver_options_default(&opt);
  const BatchParams prm = batch_params(opt);
  AFEM_TRY(batch_run(b, prm, true, ms));
  std::vector<afem_batch_result> res(b->ninst);
  AFEM_CUDA(cudaMemcpyAsync(res.data(), b->res_d, sizeof(afem_batch_result) * b->ninst, cudaMemcpyDeviceToHost,
                            b->ctx->stream));
  AFEM_CUDA(cudaStreamSynchronize(b->ctx->stream));
  if (results_h) std::copy(res.begin(), res.end(), results_h);
  for (int i = 0; i < b->ninst; ++i)
    if (res[i].status != AFEM_OK)
      return fail((afem_status)res[i].status, "afem_batch_solve: instance %d ended with status %d", i, res[i].status);
  return AFEM_OK;
}

afem_status afem_batch_autotune(afem_batch b, const afem_solver_options* opt_in, const afem_batch_config* cands,
                                int nb_cands, int reps, float* times_ms, int* best) {
  AFEM_CHECK_ARG(b && cands && nb_cands >= 1 && reps >= 1 && best, "afem_batch_autotune: bad arguments");
  afem_solver_options opt;
  if (opt_in) opt = *opt_in;
  else afem_solver_options_default(&opt);
  const BatchParams prm = batch_params(opt);
  const afem_batch_config keep = b->cfg;
  int arg = -1;
  float best_ms = 0.f;
  for (int c = 0; c < nb_cands; ++c) {
    float t = -1.f;
    afem_batch_config cfg = cands[c];
    const int occ = (cfg.block == 128 || cfg.block == 256 || cfg.block == 512) ? occupancy(cfg.block) : 0;
    if (occ >= cfg.blocks_per_sm && cfg.blocks_per_sm >= 1 && afem_batch_set_config(b, &cfg) == AFEM_OK) {
      float tmin = 0.f;
      bool ok = true;
      for (int r = 0; r < reps + 1 && ok; ++r) {   // the first run builds the graph and warms up
        float ms = 0.f;
        ok = batch_run(b, prm, true, &ms) == AFEM_OK;
        if (r == 1 || (r > 1 && ms < tmin)) tmin = ms;
      }
      if (ok) t = tmin;
    }
    if (times_ms) times_ms[c] = t;
    if (t >= 0.f && (arg < 0 || t < best_ms)) {
      arg = c;
      best_ms = t;
    }
  }
  if (arg < 0) {
    b->cfg = keep;
    batch_configure(b);
    return fail(AFEM_ERR_NOT_FOUND, "afem_batch_autotune: no candidate ran");
  }
  *best = arg;
  return afem_batch_set_config(b, &cands[arg]);
}

afem_status afem_batch_failure_test(afem_batch b, int stall_cta, long long spin_limit) {
  AFEM_CHECK_ARG(b && stall_cta >= 0 && stall_cta < b->grid && spin_limit > 0, "afem_batch_failure_test: bad arguments");
  afem_solver_options opt;
  afem_solver_options_default(&opt);
  BatchParams prm = batch_params(opt);
  prm.stall_cta = stall_cta;
  prm.spin_limit = spin_limit;
  return batch_run(b, prm, false, nullptr);
}

}  // extern "C"
