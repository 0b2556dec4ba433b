// Krylov solve on the assembled CSR system.
//
// Replaces the external HYPRE / PETSc / Aleph / Arcane MatVec solvers behind
// IDoFLinearSystemImpl::solve (femutils/HypreDoFLinearSystem.cc:596-751,
// femutils/DoFLinearSystem.cc:151-159).  Diagonal (Jacobi) preconditioned CG
// with HYPRE's two-norm stop ||r|| <= max(rtol ||b||, atol).
//
// Layout of one iteration (3 kernels, captured in a CUDA graph per chunk of
// iterations):
//   K1  q = A p, <p, q>           -> alpha        (last-block finalize)
//   K2  x += alpha p, r -= alpha q, z = D^-1 r, <r, z>, <r, r> -> beta, stop
//   K3  p = z + beta p
// Dot products are block partial sums reduced in a fixed order by the last
// block to finish (threadfence + ticket), so results are deterministic.
// A device flag stops the remaining kernels of a chunk once converged.
//
// MIXED precision: FP32 CG (FP32 matrix values and vectors; dot products in
// FP32 per thread and warp, FP64 across warps and blocks) with reliable
// updates: each time the recursive residual has fallen by inner_rtol (default
// 0.1) the FP32 correction is added to the FP64 solution, the residual is
// replaced by the true FP64 residual b - A x, and the search direction is
// KEPT (p = z + beta p with beta from the replaced residual), so the Krylov
// recurrence is not restarted.  A refinement that does not halve the true
// residual restarts the direction (p = z), and so does every refinement when
// inner_rtol < 0.01 (plain restarted refinement).  Each FP32 cycle can gain
// at most ~1 / (eps32 kappa) before the FP32 operator error floors it, which
// is why larger reductions per cycle are wasted; and with a kept direction
// the drift between recursive and true residual must stay well below the
// residual (a 1e-3 - 1e-4 reduction per cycle lost conjugacy and stalled).
#include <algorithm>
#include <cmath>

#include "afem_krylov.cuh"

namespace afem {

struct CgState {
  double rz, rr, pq, alpha, beta, bnorm2, tol2, pad0;
  int done, iter, status, max_iter;
  unsigned int ticket[4];
};

template <int G>
__global__ void __launch_bounds__(kSolveBlock) k_spmv(int n, const int32_t* __restrict__ rp,
                                                      const int32_t* __restrict__ cols, const double* __restrict__ vals,
                                                      const double* __restrict__ x, double* __restrict__ y) {
  const int lane = threadIdx.x & (G - 1);
  const int groups = gridDim.x * (blockDim.x / G);
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) / G; row < n + ((groups - n % groups) % groups);
       row += groups) {
    const bool ok = row < n;
    double s = 0.0;
    if (ok) s = row_dot<G>(row, rp, cols, vals, x, lane);
    else {
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
    }
    if (ok && lane == 0) y[row] = s;
  }
}

// r = b - A x ; z = D^-1 r ; p = z ; <r,z>, <r,r>, <b,b> (masked) ; initial stop test
template <int G>
__global__ void __launch_bounds__(kSolveBlock) k_cg_init(int n, const int32_t* __restrict__ rp,
                                                         const int32_t* __restrict__ cols,
                                                         const double* __restrict__ vals, const double* __restrict__ b,
                                                         const double* __restrict__ x, const double* __restrict__ dinv,
                                                         const uint8_t* __restrict__ skip, double* __restrict__ r,
                                                         double* __restrict__ z, double* __restrict__ p,
                                                         double* partials, CgState* st, double rtol, double atol) {
  __shared__ double sh[kSolveBlock / 32];
  const int lane = threadIdx.x & (G - 1);
  const int groups = gridDim.x * (blockDim.x / G);
  double rz = 0.0, rr = 0.0, bb = 0.0;
  const int nr = n + ((groups - n % groups) % groups);
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) / G; row < nr; row += groups) {
    double s = 0.0;
    if (row < n) s = row_dot<G>(row, rp, cols, vals, x, lane);
    else {
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
    }
    if (row < n && lane == 0) {
      double bi = b[row];
      double ri = bi - s;
      double zi = dinv ? dinv[row] * ri : ri;
      r[row] = ri;
      z[row] = zi;
      p[row] = zi;
      rz += ri * zi;
      if (!(skip && skip[row])) {
        rr += ri * ri;
        bb += bi * bi;
      }
    }
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  bb = block_sum(bb, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x * 3 + 0] = rz;
    partials[blockIdx.x * 3 + 1] = rr;
    partials[blockIdx.x * 3 + 2] = bb;
  }
  if (last_block(&st->ticket[0])) {
    double trz = reduce_partials(partials, gridDim.x, 3, 0, sh);
    double trr = reduce_partials(partials, gridDim.x, 3, 1, sh);
    double tbb = reduce_partials(partials, gridDim.x, 3, 2, sh);
    if (threadIdx.x == 0) {
      st->rz = trz;
      st->rr = trr;
      st->bnorm2 = tbb;
      double t = std::max(rtol * rtol * tbb, atol * atol);
      st->tol2 = t;
      st->iter = 0;
      st->status = AFEM_OK;
      st->done = (trr <= t) ? 1 : 0;
      st->ticket[0] = 0;
    }
  }
}

// K1 (q = A p, <p, q> -> alpha) is k_cg_spmv_sl, over the sliced-ELL copy below.

// K2: x += alpha p ; r -= alpha q ; z = D^-1 r ; <r,z>, <r,r> -> beta, stop test
__global__ void __launch_bounds__(kSolveBlock) k_cg_update(int n, double* __restrict__ x, double* __restrict__ r,
                                                           double* __restrict__ z, const double* __restrict__ p,
                                                           const double* __restrict__ q,
                                                           const double* __restrict__ dinv,
                                                           const uint8_t* __restrict__ skip, double* partials,
                                                           CgState* st) {
  if (((volatile CgState*)st)->done) return;
  __shared__ double sh[kSolveBlock / 32];
  const double alpha = ((volatile CgState*)st)->alpha;
  double rz = 0.0, rr = 0.0;
  // two elements per thread and pass (16-byte accesses: every vector here is
  // one of the solver's own 256-byte-aligned buffers), then the odd tail
  const int n2 = n >> 1;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int i = tid; i < n2; i += stride) {
    const double2 pv = reinterpret_cast<const double2*>(p)[i], qv = reinterpret_cast<const double2*>(q)[i];
    double2 xv = reinterpret_cast<double2*>(x)[i], rv = reinterpret_cast<double2*>(r)[i];
    xv.x += alpha * pv.x;
    xv.y += alpha * pv.y;
    rv.x = rv.x - alpha * qv.x;
    rv.y = rv.y - alpha * qv.y;
    double2 zv = rv;
    if (dinv) {
      const double2 dv = reinterpret_cast<const double2*>(dinv)[i];
      zv = make_double2(dv.x * rv.x, dv.y * rv.y);
    }
    reinterpret_cast<double2*>(x)[i] = xv;
    reinterpret_cast<double2*>(r)[i] = rv;
    reinterpret_cast<double2*>(z)[i] = zv;
    rz += rv.x * zv.x;
    rz += rv.y * zv.y;
    if (!(skip && skip[2 * i])) rr += rv.x * rv.x;
    if (!(skip && skip[2 * i + 1])) rr += rv.y * rv.y;
  }
  for (int i = 2 * n2 + tid; i < n; i += stride) {
    double pi = p[i];
    x[i] += alpha * pi;
    double ri = r[i] - alpha * q[i];
    r[i] = ri;
    double zi = dinv ? dinv[i] * ri : ri;
    z[i] = zi;
    rz += ri * zi;
    if (!(skip && skip[i])) rr += ri * ri;
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x * 2 + 0] = rz;
    partials[blockIdx.x * 2 + 1] = rr;
  }
  if (last_block(&st->ticket[2])) {
    double trz = reduce_partials(partials, gridDim.x, 2, 0, sh);
    double trr = reduce_partials(partials, gridDim.x, 2, 1, sh);
    if (threadIdx.x == 0) {
      st->beta = trz / st->rz;
      st->rz = trz;
      st->rr = trr;
      st->iter += 1;
      if (!isfinite(trr)) {
        st->status = AFEM_ERR_BREAKDOWN;
        st->done = 1;
      } else if (trr <= st->tol2) {
        st->done = 1;
      } else if (st->iter >= st->max_iter) {
        st->status = AFEM_ERR_NOT_CONVERGED;
        st->done = 1;
      }
      st->ticket[2] = 0;
    }
  }
}

// K3: p = z + beta p (skipped once converged: p is not used any more)
__global__ void __launch_bounds__(kSolveBlock) k_cg_dir(int n, const double* __restrict__ z, double* __restrict__ p,
                                                        const CgState* st) {
  if (((volatile const CgState*)st)->done) return;
  const double beta = ((volatile const CgState*)st)->beta;
  const int n2 = n >> 1;   // 16-byte accesses (solver-owned aligned buffers), then the tail
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int i = tid; i < n2; i += stride) {
    const double2 zv = reinterpret_cast<const double2*>(z)[i];
    double2 pv = reinterpret_cast<double2*>(p)[i];
    pv = make_double2(zv.x + beta * pv.x, zv.y + beta * pv.y);
    reinterpret_cast<double2*>(p)[i] = pv;
  }
  for (int i = 2 * n2 + tid; i < n; i += stride) p[i] = z[i] + beta * p[i];
}

// D^-1 from the diagonal entries (1 where the diagonal is missing or zero).
__global__ void k_inv_diag(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                           const double* __restrict__ vals, double* __restrict__ dinv, float* __restrict__ dinv32) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
      if (cols[k] == i) {
        d = vals[k];
        break;
      }
    double v = d != 0.0 ? 1.0 / d : 1.0;
    if (dinv) dinv[i] = v;
    if (dinv32) dinv32[i] = (float)v;
  }
}

// ---------------------------------------------------------------------------
// FP32 inner CG (mixed precision).  Same structure, FP32 vectors and values;
// dot products accumulate in FP32 per thread and warp, in FP64 across warps
// and blocks.

// FP64 CG K1 over the sliced copy: q = A p, <p, q> -> alpha (the breakdown test as k_cgf_spmv_sl;
// each row's products are added in CSR order, as in row_dot_chunked)
__global__ void __launch_bounds__(kSolveBlock) k_cg_spmv_sl(int n, const int32_t* __restrict__ soff,
                                                            const int32_t* __restrict__ scols,
                                                            const double* __restrict__ svals,
                                                            const double* __restrict__ p, double* __restrict__ q,
                                                            double* partials, CgState* st) {
  if (((volatile CgState*)st)->done) return;
  __shared__ double sh[kSolveBlock / 32];
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;   // a multiple of 32: a warp is one slice
  const int64_t nr = ((int64_t)n + kSlice - 1) / kSlice * kSlice;
  double pq = 0.0;
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < nr; row += stride) {
    const int64_t sl = row / kSlice;
    const int m = __ldg(soff + sl + 1) - __ldg(soff + sl);
    const int32_t* c = scols + (int64_t)kSlice * __ldg(soff + sl) + (row & (kSlice - 1));
    const double acc = sliced_row_dot<double>(c, svals + (c - scols), m, p);
    if (row < n) {
      q[row] = acc;
      pq += p[row] * acc;
    }
  }
  pq = block_sum(pq, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = pq;
  if (last_block(&st->ticket[1])) {
    double t = reduce_partials(partials, gridDim.x, 1, 0, sh);
    if (threadIdx.x == 0) {
      st->pq = t;
      if (!(t > 0.0) || !isfinite(t)) {
        st->status = AFEM_ERR_BREAKDOWN;
        st->done = 1;
        st->alpha = 0.0;
      } else {
        st->alpha = st->rz / t;
      }
      st->ticket[1] = 0;
    }
  }
}

// Inner CG step K1, fused with the direction update of the previous step:
//   w = A z ; p = z + beta p ; q = w + beta q (= A p) ; <p, q> -> alpha
// over the sliced copy.  The SpMV reads z only, so p and q are updated in
// place for the thread's own rows.  beta = 0 (first step of a cycle, or a
// restarted direction) gives p = z, q = A z without reading the old p and q.
// q follows the recurrence A z + beta q instead of a product with p; the
// reliable FP64 updates every cycle bound the drift of both.
__global__ void __launch_bounds__(kSolveBlock) k_cgf_spmv_sl(int n, const int32_t* __restrict__ soff,
                                                             const int32_t* __restrict__ scols,
                                                             const float* __restrict__ svals,
                                                             const float* __restrict__ z, float* __restrict__ p,
                                                             float* __restrict__ q, double* partials, CgState* st) {
  if (((volatile CgState*)st)->done) return;
  __shared__ double sh[kSolveBlock / 32];
  const float beta = (float)((volatile CgState*)st)->beta;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;   // a multiple of 32: a warp is one slice
  const int64_t nr = ((int64_t)n + kSlice - 1) / kSlice * kSlice;
  float pqf = 0.f;
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < nr; row += stride) {
    const int64_t sl = row / kSlice;
    const int m = __ldg(soff + sl + 1) - __ldg(soff + sl);
    const int32_t* c = scols + (int64_t)kSlice * __ldg(soff + sl) + (row & (kSlice - 1));
    const float w = sliced_row_dot<float>(c, svals + (c - scols), m, z);
    if (row < n) {
      const float zi = z[row];
      const float pi = beta != 0.f ? fmaf(beta, p[row], zi) : zi;
      const float qi = beta != 0.f ? fmaf(beta, q[row], w) : w;
      p[row] = pi;
      q[row] = qi;
      pqf = fmaf(pi, qi, pqf);
    }
  }
  const double pq = block_sum_f(pqf, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = pq;
  if (last_block(&st->ticket[1])) {
    double t = reduce_partials(partials, gridDim.x, 1, 0, sh);
    if (threadIdx.x == 0) {
      st->pq = t;
      if (!(t > 0.0) || !isfinite(t)) {
        st->status = AFEM_ERR_BREAKDOWN;
        st->done = 1;
        st->alpha = 0.0;
      } else {
        st->alpha = st->rz / t;
      }
      st->ticket[1] = 0;
    }
  }
}

// Block columns of a CSR whose scalar rows come in 3x3 blocks (the per-row
// layout of a 3-DoF BSR matrix, femutils/BSRFormat.h: block row I = scalar
// rows 3I..3I+2 with one pattern, columns 3J..3J+2 per block): one index per
// block, and *bad set if the pattern is not of that form.
__global__ void k_block_cols3(int nb, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                              int32_t* __restrict__ bcols, int* __restrict__ bad) {
  for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < nb; I += gridDim.x * blockDim.x) {
    const int32_t r0 = rp[3 * I], len = rp[3 * I + 1] - r0;
    if (len % 3 != 0 || r0 % 9 != 0 || rp[3 * I + 2] - rp[3 * I + 1] != len || rp[3 * I + 3] - rp[3 * I + 2] != len) {
      atomicOr(bad, 1);
      continue;
    }
    for (int32_t k = 0; k < len; k += 3) {
      const int32_t c = cols[r0 + k];
      bool ok = c % 3 == 0;
      for (int a = 0; a < 3 && ok; ++a)
        for (int b = 0; b < 3 && ok; ++b) ok = cols[r0 + a * len + k + b] == c + b;
      if (!ok) {
        atomicOr(bad, 1);
        break;
      }
      bcols[r0 / 9 + k / 3] = c / 3;
    }
  }
}

// Sliced copy of a 3x3-block matrix for the FP32 SpMV: 32 block rows per
// slice, padded to the slice's longest block row; block kb of block row
// 32 s + l has its column index at 32 bsoff[s] + 32 kb + l and its value
// (a, b) at (32 bsoff[s] + 32 kb) * 9 + (3 a + b) * 32 + l.  Warp (s, a)
// computes the scalar rows 3 (32 s + l) + a: per block one coalesced
// 128-byte segment of block columns (shared by the slice's three warps) and
// three of values.  Padding blocks are zero blocks on the row's own block
// column.  Each scalar row adds its products block by block, b inner, the
// order of a thread-per-row walk of the block CSR rows, so q is unchanged;
// <p, q> accumulates its rows in another order (warps own slices).
constexpr int kB3Chunk = 3;   // blocks per chunk of loads issued before their products

__global__ void k_slice_len3(int nb, const int32_t* __restrict__ rp, int32_t* __restrict__ slen) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nr = ((int64_t)nb + kSlice - 1) / kSlice * kSlice;
  for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < nr; I += stride) {
    const int len = I < nb ? (__ldg(rp + 3 * I + 1) - __ldg(rp + 3 * I)) / 3 : 0;
    const int m = __reduce_max_sync(0xffffffffu, len);
    if ((I & (kSlice - 1)) == 0) slen[I / kSlice] = m;
  }
}

__global__ void k_slice_fill3(int nb, const int32_t* __restrict__ rp, const int32_t* __restrict__ bcols,
                              const double* __restrict__ vals, const int32_t* __restrict__ soff,
                              int32_t* __restrict__ scols, float* __restrict__ svals) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nr = ((int64_t)nb + kSlice - 1) / kSlice * kSlice;
  for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < nr; I += stride) {
    const int64_t sl = I / kSlice, l = I & (kSlice - 1);
    const int m = soff[sl + 1] - soff[sl];
    const int32_t r0 = I < nb ? rp[3 * I] : 0;
    const int nbk = I < nb ? (rp[3 * I + 1] - r0) / 3 : 0;
    for (int kb = 0; kb < m; ++kb) {
      const bool in = kb < nbk;
      const int64_t e = (int64_t)kSlice * soff[sl] + (int64_t)kSlice * kb;
      scols[e + l] = in ? bcols[r0 / 9 + kb] : (I < nb ? (int32_t)I : 0);
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b)
          svals[e * 9 + (3 * a + b) * kSlice + l] = in ? (float)vals[rp[3 * I + a] + 3 * kb + b] : 0.f;
    }
  }
}

// K1 of the inner CG over the block slices, fused with the direction update
// as k_cgf_spmv_sl: w = A z gathered by blocks, then p and q in place.
__global__ void __launch_bounds__(kSolveBlock) k_cgf_spmv_b3s(int nb, const int32_t* __restrict__ soff,
                                                              const int32_t* __restrict__ scols,
                                                              const float* __restrict__ svals,
                                                              const float* __restrict__ z, float* __restrict__ p,
                                                              float* __restrict__ q, double* partials, CgState* st) {
  if (((volatile CgState*)st)->done) return;
  __shared__ double sh[kSolveBlock / 32];
  const float beta = (float)((volatile CgState*)st)->beta;
  const int lane = threadIdx.x & 31;
  const int64_t nslice = ((int64_t)nb + kSlice - 1) / kSlice;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x / 32);
  float pqf = 0.f;
  for (int64_t w = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / 32; w < 3 * nslice; w += warps) {
    const int64_t sl = w / 3;
    const int a = (int)(w - 3 * sl);
    const int m = __ldg(soff + sl + 1) - __ldg(soff + sl);
    const int64_t e0 = (int64_t)kSlice * __ldg(soff + sl);
    const int32_t* c = scols + e0 + lane;
    const float* v = svals + e0 * 9 + 3 * a * kSlice + lane;
    // chunks of kB3Chunk blocks, all loads first (past the row's end they read its first block), products past
    // the end skipped by a warp-uniform branch
    float acc = 0.f;
    for (int kb = 0; kb < m; kb += kB3Chunk) {
      int32_t j[kB3Chunk];
      float x[3 * kB3Chunk];
#pragma unroll
      for (int u = 0; u < kB3Chunk; ++u) {
        const int e = kb + u < m ? kb + u : 0;
        j[u] = 3 * __ldg(c + (int64_t)kSlice * e);
#pragma unroll
        for (int b = 0; b < 3; ++b) x[3 * u + b] = __ldg(v + (int64_t)kSlice * 9 * e + b * kSlice);
      }
#pragma unroll
      for (int u = 0; u < kB3Chunk; ++u)
        if (kb + u < m)
#pragma unroll
          for (int b = 0; b < 3; ++b) acc = fmaf(x[3 * u + b], __ldg(z + j[u] + b), acc);
    }
    const int64_t I = kSlice * sl + lane;
    if (I < nb) {
      const int64_t row = 3 * I + a;
      const float zi = z[row];
      const float pi = beta != 0.f ? fmaf(beta, p[row], zi) : zi;
      const float qi = beta != 0.f ? fmaf(beta, q[row], acc) : acc;
      p[row] = pi;
      q[row] = qi;
      pqf = fmaf(pi, qi, pqf);
    }
  }
  const double pq = block_sum_f(pqf, sh);
  if (threadIdx.x == 0) partials[blockIdx.x] = pq;
  if (last_block(&st->ticket[1])) {
    double t = reduce_partials(partials, gridDim.x, 1, 0, sh);
    if (threadIdx.x == 0) {
      st->pq = t;
      if (!(t > 0.0) || !isfinite(t)) {
        st->status = AFEM_ERR_BREAKDOWN;
        st->done = 1;
        st->alpha = 0.0;
      } else {
        st->alpha = st->rz / t;
      }
      st->ticket[1] = 0;
    }
  }
}

__global__ void __launch_bounds__(kSolveBlock) k_cgf_update(int n, float* __restrict__ x, float* __restrict__ r,
                                                            float* __restrict__ z, const float* __restrict__ p,
                                                            const float* __restrict__ q,
                                                            const float* __restrict__ dinv,
                                                            const uint8_t* __restrict__ skip, double* partials,
                                                            CgState* st) {
  if (((volatile CgState*)st)->done) return;
  __shared__ double sh[kSolveBlock / 32];
  const float alpha = (float)((volatile CgState*)st)->alpha;
  float rzf = 0.f, rrf = 0.f;
  // four elements per thread and pass (16-byte accesses: the vectors are the
  // solver's own 256-byte-aligned buffers), then the n % 4 tail
  const int n4 = n >> 2;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int i = tid; i < n4; i += stride) {
    const float4 pv = reinterpret_cast<const float4*>(p)[i], qv = reinterpret_cast<const float4*>(q)[i];
    const float4 dv = reinterpret_cast<const float4*>(dinv)[i];
    float4 xv = reinterpret_cast<float4*>(x)[i], rv = reinterpret_cast<float4*>(r)[i];
    xv.x = fmaf(alpha, pv.x, xv.x);
    xv.y = fmaf(alpha, pv.y, xv.y);
    xv.z = fmaf(alpha, pv.z, xv.z);
    xv.w = fmaf(alpha, pv.w, xv.w);
    rv.x = fmaf(-alpha, qv.x, rv.x);
    rv.y = fmaf(-alpha, qv.y, rv.y);
    rv.z = fmaf(-alpha, qv.z, rv.z);
    rv.w = fmaf(-alpha, qv.w, rv.w);
    const float4 zv = make_float4(dv.x * rv.x, dv.y * rv.y, dv.z * rv.z, dv.w * rv.w);
    reinterpret_cast<float4*>(x)[i] = xv;
    reinterpret_cast<float4*>(r)[i] = rv;
    reinterpret_cast<float4*>(z)[i] = zv;
    rzf = fmaf(rv.x, zv.x, rzf);
    rzf = fmaf(rv.y, zv.y, rzf);
    rzf = fmaf(rv.z, zv.z, rzf);
    rzf = fmaf(rv.w, zv.w, rzf);
    const int e = 4 * i;
    if (!(skip && skip[e])) rrf = fmaf(rv.x, rv.x, rrf);
    if (!(skip && skip[e + 1])) rrf = fmaf(rv.y, rv.y, rrf);
    if (!(skip && skip[e + 2])) rrf = fmaf(rv.z, rv.z, rrf);
    if (!(skip && skip[e + 3])) rrf = fmaf(rv.w, rv.w, rrf);
  }
  for (int i = 4 * n4 + tid; i < n; i += stride) {
    x[i] = fmaf(alpha, p[i], x[i]);
    float ri = fmaf(-alpha, q[i], r[i]);
    r[i] = ri;
    float zi = dinv[i] * ri;
    z[i] = zi;
    rzf = fmaf(ri, zi, rzf);
    if (!(skip && skip[i])) rrf = fmaf(ri, ri, rrf);
  }
  const double rz = block_sum_f(rzf, sh);
  const double rr = block_sum_f(rrf, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x * 2 + 0] = rz;
    partials[blockIdx.x * 2 + 1] = rr;
  }
  if (last_block(&st->ticket[2])) {
    double trz = reduce_partials(partials, gridDim.x, 2, 0, sh);
    double trr = reduce_partials(partials, gridDim.x, 2, 1, sh);
    if (threadIdx.x == 0) {
      st->beta = trz / st->rz;
      st->pad0 = st->rz;   // <r, z> before this step, for a reliable update that keeps p
      st->rz = trz;
      st->rr = trr;
      st->iter += 1;
      if (!isfinite(trr)) {
        st->status = AFEM_ERR_BREAKDOWN;
        st->done = 1;
      } else if (trr <= st->tol2 || st->iter >= st->max_iter) {
        st->done = 1;
      }
      st->ticket[2] = 0;
    }
  }
}


// Reliable update: r = b - A x (FP64), r32 = (float) r, x32 = 0,
// z32 = D^-1 r32 ; <r32, z32> and FP64 ||r||^2 ; inner state reset.  The
// inner state's beta is 0 with `restart` (the next K1 starts p = z), else
// <r32, z32> / <r, z>_prev (the next K1 keeps the direction: p = z + beta p).
template <int G>
__global__ void __launch_bounds__(kSolveBlock) k_ir_residual(
    int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols, const double* __restrict__ vals,
    const double* __restrict__ b, const double* __restrict__ x, const float* __restrict__ dinv32,
    const uint8_t* __restrict__ skip, float* __restrict__ r32, float* __restrict__ x32, float* __restrict__ z32,
    double* partials, CgState* outer, CgState* inner, double inner_rtol, int inner_max, int restart) {
  __shared__ double sh[kSolveBlock / 32];
  const int lane = threadIdx.x & (G - 1);
  const int groups = gridDim.x * (blockDim.x / G);
  const int nr = n + ((groups - n % groups) % groups);
  double rz = 0.0, rr = 0.0, bb = 0.0;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) / G; row < nr; row += groups) {
    double s = 0.0;
    if (row < n) s = row_dot<G>(row, rp, cols, vals, x, lane);
    else {
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
    }
    if (row < n && lane == 0) {
      double bi = b[row];
      double ri = bi - s;
      float rf = (float)ri;
      float zf = dinv32[row] * rf;
      r32[row] = rf;
      x32[row] = 0.f;
      z32[row] = zf;
      rz += (double)rf * (double)zf;
      if (!(skip && skip[row])) {
        rr += ri * ri;
        bb += bi * bi;
      }
    }
  }
  rz = block_sum(rz, sh);
  rr = block_sum(rr, sh);
  bb = block_sum(bb, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x * 3 + 0] = rz;
    partials[blockIdx.x * 3 + 1] = rr;
    partials[blockIdx.x * 3 + 2] = bb;
  }
  if (last_block(&outer->ticket[0])) {
    double trz = reduce_partials(partials, gridDim.x, 3, 0, sh);
    double trr = reduce_partials(partials, gridDim.x, 3, 1, sh);
    double tbb = reduce_partials(partials, gridDim.x, 3, 2, sh);
    if (threadIdx.x == 0) {
      outer->rr = trr;
      outer->bnorm2 = tbb;
      outer->done = (trr <= outer->tol2) ? 1 : 0;
      outer->ticket[0] = 0;
      inner->beta = restart ? 0.0 : trz / inner->pad0;
      inner->rz = trz;
      inner->rr = trr;
      inner->tol2 = inner_rtol * inner_rtol * trr;
      inner->iter = 0;
      inner->max_iter = inner_max;
      inner->status = AFEM_OK;
      inner->done = outer->done;
    }
  }
}


__global__ void k_ir_correct(int n, double* __restrict__ x, const float* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += (double)d[i];
}


__global__ void k_fill_f32(int64_t n, float v, float* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = v;
}

// ---------------------------------------------------------------------------
// Host side.

// Sliced copy of a validated 3x3-block matrix (block columns from k_block_cols3)
static afem_status build_slices3(afem_context ctx, int nb, const int32_t* rp, const int32_t* bcols,
                                 const double* vals, SlicedCopy<float>& out) {
  out.release();
  out.s = ctx->stream;
  out.n = nb;
  const int64_t nslice = ((int64_t)nb + kSlice - 1) / kSlice;
  int32_t* slen;
  AFEM_TRY(scratch_take(ctx, (size_t)nslice + 1, &slen));
  AFEM_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&out.soff), sizeof(int32_t) * (size_t)(nslice + 1), ctx->stream));
  AFEM_TRY(launch(ctx, k_slice_len3, grid_for(ctx, nslice * kSlice, 256), 256, 0, nb, rp, slen));
  AFEM_TRY(exclusive_scan_i32(ctx, slen, out.soff, nslice));
  int32_t slots = 0;   // sum of the slice lengths in blocks (<= nnz / 9)
  AFEM_TRY(read_scalar(ctx, out.soff + nslice, &slots));
  const size_t entries = (size_t)kSlice * (size_t)std::max(slots, 1);
  AFEM_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&out.cols), sizeof(int32_t) * entries, ctx->stream));
  AFEM_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&out.vals), sizeof(float) * 9 * entries, ctx->stream));
  return launch(ctx, k_slice_fill3, grid_for(ctx, nslice * kSlice, 256), 256, 0, nb, rp, bcols, vals,
                (const int32_t*)out.soff, out.cols, out.vals);
}

afem_status cg_fp64(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals, int64_t nnz,
                    const double* b, double* x, const uint8_t* skip, const afem_solver_options& opt,
                    afem_solve_info* info) {
  const int G = lanes_per_row_fp64(n, nnz);
  const unsigned grid_rows = grid_for(ctx, (int64_t)n * G, kSolveBlock, 8);
  const unsigned grid_vec = grid_for(ctx, n, kSolveBlock, 8);
  const unsigned nparts = std::max(grid_rows, grid_vec);
  size_t need = 6 * align256(sizeof(double) * (size_t)n) + align256(sizeof(double) * 3 * nparts) +
                align256(sizeof(CgState)) + slices_scratch_bytes(n);
  AFEM_TRY(scratch_reserve(ctx, need));
  double *r, *z, *p, *q, *dinv, *partials;
  CgState* st;
  // the iterate lives in an aligned scratch copy (16-byte vector accesses in
  // k_cg_update), copied in here and back to the caller's x at the end
  double* const x_user = x;
  AFEM_TRY(scratch_take(ctx, n, &x));
  AFEM_CUDA(cudaMemcpyAsync(x, x_user, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
  AFEM_TRY(scratch_take(ctx, n, &r));
  AFEM_TRY(scratch_take(ctx, n, &z));
  AFEM_TRY(scratch_take(ctx, n, &p));
  AFEM_TRY(scratch_take(ctx, n, &q));
  AFEM_TRY(scratch_take(ctx, n, &dinv));
  AFEM_TRY(scratch_take(ctx, 3 * (size_t)nparts, &partials));
  AFEM_TRY(scratch_take(ctx, 1, &st));
  AFEM_CUDA(cudaMemsetAsync(st, 0, sizeof(CgState), ctx->stream));
  const int max_iter = opt.max_iter > 0 ? opt.max_iter : 1000;
  AFEM_CUDA(cudaMemcpyAsync(&st->max_iter, &max_iter, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  const bool jacobi = opt.precond == AFEM_PRECOND_JACOBI;
  if (jacobi)
    AFEM_TRY(launch(ctx, k_inv_diag, grid_vec, kSolveBlock, 0, n, rp, cols, vals, dinv, (float*)nullptr));
  const double* dv = jacobi ? dinv : nullptr;
  AFEM_TRY(dispatch_g(G, [&](auto g) {
    return launch(ctx, k_cg_init<decltype(g)::value>, grid_rows, kSolveBlock, 0, n, rp, cols, vals, b,
                  (const double*)x, dv, skip, r, z, p, partials, st, opt.rtol, opt.atol);
  }));
  SlicedCopy<double> sliced;   // the iteration's SpMV reads the sliced-ELL copy
  AFEM_TRY(build_slices(ctx, n, rp, cols, vals, sliced));
  const unsigned grid_sl = grid_for(ctx, n, kSolveBlock, 8);
  const int chunk = opt.check_every > 0 ? opt.check_every : 16;
  GraphChunk gc;
  AFEM_TRY(capture(ctx, gc, [&](cudaStream_t s) -> afem_status {
    for (int k = 0; k < chunk; ++k) {
      AFEM_TRY(launch_s(ctx, s, k_cg_spmv_sl, grid_sl, kSolveBlock, n, (const int32_t*)sliced.soff,
                        (const int32_t*)sliced.cols, (const double*)sliced.vals, (const double*)p, q, partials, st));
      AFEM_TRY(launch_s(ctx, s, k_cg_update, grid_vec, kSolveBlock, n, x, r, z, (const double*)p, (const double*)q,
                        dv, skip, partials, st));
      AFEM_TRY(launch_s(ctx, s, k_cg_dir, grid_vec, kSolveBlock, n, (const double*)z, p, (const CgState*)st));
    }
    return AFEM_OK;
  }));
  CgState hs{};
  for (int done_chunks = 0;; ++done_chunks) {
    AFEM_CUDA(cudaMemcpyAsync(ctx->pinned, st, sizeof(CgState), cudaMemcpyDeviceToHost, ctx->stream));
    AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
    hs = *reinterpret_cast<CgState*>(ctx->pinned);
    if (hs.done) break;
    AFEM_CUDA(cudaGraphLaunch(gc.exec, ctx->stream));
    ctx->launches += 3 * chunk;
  }
  AFEM_CUDA(cudaMemcpyAsync(x_user, x, sizeof(double) * (size_t)n, cudaMemcpyDeviceToDevice, ctx->stream));
  if (info) {
    info->iterations = hs.iter;
    info->refinements = 0;
    info->status = hs.status;
  }
  return hs.status;
}

afem_status cg_mixed(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals, int64_t nnz,
                     const double* b, double* x, const uint8_t* skip, const afem_solver_options& opt,
                     afem_solve_info* info) {
  const int G64 = lanes_per_row_fp64(n, nnz);   // FP64 outer residual
  const bool b3 = opt.block_size == 3;          // FP32 3x3-block SpMV, else the sliced-ELL scalar SpMV
  AFEM_CHECK_ARG(!b3 || n % 3 == 0, "block_size 3 needs a multiple of 3 rows (%d)", n);
  const unsigned grid_rows = grid_for(ctx, n, kSolveBlock, 8);
  const unsigned grid_rows64 = grid_for(ctx, (int64_t)n * G64, kSolveBlock, 8);
  const unsigned grid_vec = grid_for(ctx, n, kSolveBlock, 8);
  // 3x3-block SpMV: one warp per (slice of 32 block rows, component)
  const unsigned grid_b3 = grid_for(ctx, 3 * (((int64_t)n / 3 + kSlice - 1) / kSlice) * kSlice, kSolveBlock, 8);
  const unsigned nparts = std::max(std::max(std::max(grid_rows, grid_rows64), grid_vec), grid_b3);
  size_t need = 6 * align256(sizeof(float) * (size_t)n) + align256(sizeof(double) * 3 * nparts) +
                2 * align256(sizeof(CgState)) +
                (b3 ? align256(sizeof(int32_t) * (size_t)(nnz / 9 + 1)) + 256 + slices_scratch_bytes(n / 3)
                    : slices_scratch_bytes(n));
  AFEM_TRY(scratch_reserve(ctx, need));
  float *r32, *z32, *p32, *q32, *x32, *dinv32;
  double* partials;
  CgState *outer, *inner;
  AFEM_TRY(scratch_take(ctx, n, &r32));
  AFEM_TRY(scratch_take(ctx, n, &z32));
  AFEM_TRY(scratch_take(ctx, n, &p32));
  AFEM_TRY(scratch_take(ctx, n, &q32));
  AFEM_TRY(scratch_take(ctx, n, &x32));
  AFEM_TRY(scratch_take(ctx, n, &dinv32));
  AFEM_TRY(scratch_take(ctx, 3 * (size_t)nparts, &partials));
  AFEM_TRY(scratch_take(ctx, 1, &outer));
  AFEM_TRY(scratch_take(ctx, 1, &inner));
  AFEM_CUDA(cudaMemsetAsync(outer, 0, sizeof(CgState), ctx->stream));
  AFEM_CUDA(cudaMemsetAsync(inner, 0, sizeof(CgState), ctx->stream));
  int32_t* bcols = nullptr;
  if (b3) {
    int* bad;
    AFEM_TRY(scratch_take(ctx, (size_t)(nnz / 9 + 1), &bcols));
    AFEM_TRY(scratch_take(ctx, 1, &bad));
    AFEM_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
    AFEM_TRY(launch(ctx, k_block_cols3, grid_for(ctx, n / 3, 256), 256, 0, n / 3, rp, cols, bcols, bad));
    int hbad = 0;
    AFEM_TRY(read_scalar(ctx, bad, &hbad));
    AFEM_CHECK_ARG(!hbad, "block_size 3: the CSR pattern is not made of 3x3 blocks");
  }
  // the FP32 matrix: the sliced copy, by 3x3 blocks or by scalar rows
  SlicedCopy<float> sliced;
  if (b3)
    AFEM_TRY(build_slices3(ctx, n / 3, rp, (const int32_t*)bcols, vals, sliced));
  else
    AFEM_TRY(build_slices(ctx, n, rp, cols, vals, sliced));
  AFEM_TRY(launch(ctx, k_inv_diag, grid_vec, kSolveBlock, 0, n, rp, cols, vals, (double*)nullptr, dinv32));
  if (opt.precond != AFEM_PRECOND_JACOBI)  // unpreconditioned inner solve: D^-1 = 1
    AFEM_TRY(launch(ctx, k_fill_f32, grid_for(ctx, n, 256), 256, 0, (int64_t)n, 1.0f, dinv32));
  const double inner_rtol = opt.inner_rtol > 0 ? opt.inner_rtol : 0.1;
  const int max_iter = opt.max_iter > 0 ? opt.max_iter : 1000;
  const int chunk = opt.check_every > 0 ? opt.check_every : 16;
  // outer tolerance: needs ||b||, computed by the first residual pass
  GraphChunk gc;
  AFEM_TRY(capture(ctx, gc, [&](cudaStream_t s) -> afem_status {
    for (int k = 0; k < chunk; ++k) {
      if (b3)
        AFEM_TRY(launch_s(ctx, s, k_cgf_spmv_b3s, grid_b3, kSolveBlock, n / 3, (const int32_t*)sliced.soff,
                          (const int32_t*)sliced.cols, (const float*)sliced.vals, (const float*)z32, p32, q32,
                          partials, inner));
      else
        AFEM_TRY(launch_s(ctx, s, k_cgf_spmv_sl, grid_rows, kSolveBlock, n, (const int32_t*)sliced.soff,
                          (const int32_t*)sliced.cols, (const float*)sliced.vals, (const float*)z32, p32, q32,
                          partials, inner));
      AFEM_TRY(launch_s(ctx, s, k_cgf_update, grid_vec, kSolveBlock, n, x32, r32, z32, (const float*)p32,
                        (const float*)q32, (const float*)dinv32, skip, partials, inner));
    }
    return AFEM_OK;
  }));
  int total_inner = 0, outer_steps = 0;
  afem_status status = AFEM_OK;
  const int max_outer = 1000;
  double rr_prev = 0.0;      // true ||r||^2 at the previous update
  bool restart = true;
  for (;; ++outer_steps) {
    // max_iter bounds the inner iterations of the whole solve (the reference's
    // max-iter, HypreDoFLinearSystem.cc:182): each cycle gets what remains
    const int remaining = std::max(1, max_iter - total_inner);
    AFEM_TRY(dispatch_g(G64, [&](auto g) {
      return launch(ctx, k_ir_residual<decltype(g)::value>, grid_rows64, kSolveBlock, 0, n, rp, cols, vals, b,
                    (const double*)x, (const float*)dinv32, skip, r32, x32, z32, partials, outer, inner,
                    inner_rtol, remaining, restart ? 1 : 0);
    }));
    CgState ho{};
    AFEM_CUDA(cudaMemcpyAsync(ctx->pinned, outer, sizeof(CgState), cudaMemcpyDeviceToHost, ctx->stream));
    AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
    ho = *reinterpret_cast<CgState*>(ctx->pinned);
    if (!restart && !(ho.rr <= 0.25 * rr_prev && inner_rtol >= 0.01)) {
      // the true residual did not halve: redo this update with a fresh direction
      restart = true;
      AFEM_TRY(dispatch_g(G64, [&](auto g) {
        return launch(ctx, k_ir_residual<decltype(g)::value>, grid_rows64, kSolveBlock, 0, n, rp, cols, vals, b,
                      (const double*)x, (const float*)dinv32, skip, r32, x32, z32, partials, outer, inner,
                      inner_rtol, remaining, 1);
      }));
      AFEM_CUDA(cudaMemcpyAsync(ctx->pinned, outer, sizeof(CgState), cudaMemcpyDeviceToHost, ctx->stream));
      AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
      ho = *reinterpret_cast<CgState*>(ctx->pinned);
    }
    rr_prev = ho.rr;
    restart = false;
    if (outer_steps == 0) {
      // first pass: set the FP64 outer tolerance from ||b|| and re-test
      double tol2 = std::max(opt.rtol * opt.rtol * ho.bnorm2, opt.atol * opt.atol);
      ho.tol2 = tol2;
      AFEM_CUDA(cudaMemcpyAsync(&outer->tol2, &ho.tol2, sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
      if (ho.rr <= tol2) break;
      int d = 0;
      AFEM_CUDA(cudaMemcpyAsync(&inner->done, &d, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    } else if (ho.done) {
      break;
    }
    if (outer_steps >= max_outer || total_inner >= max_iter) {
      status = AFEM_ERR_NOT_CONVERGED;
      break;
    }
    CgState hi{};
    for (;;) {
      AFEM_CUDA(cudaGraphLaunch(gc.exec, ctx->stream));
      ctx->launches += 2 * chunk;
      AFEM_CUDA(cudaMemcpyAsync(ctx->pinned, inner, sizeof(CgState), cudaMemcpyDeviceToHost, ctx->stream));
      AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
      hi = *reinterpret_cast<CgState*>(ctx->pinned);
      if (hi.done) break;
    }
    total_inner += hi.iter;
    if (hi.status == AFEM_ERR_BREAKDOWN && hi.iter == 0) {
      status = AFEM_ERR_BREAKDOWN;
      break;
    }
    AFEM_TRY(launch(ctx, k_ir_correct, grid_vec, 256, 0, n, x, (const float*)x32));
  }
  if (info) {
    info->iterations = total_inner;
    info->refinements = outer_steps;
    info->status = status;
  }
  return status;
}

// ||b - A x||^2 and ||b||^2 (masked), FP64, written to out[0], out[1].
template <int G>
__global__ void __launch_bounds__(kSolveBlock) k_true_residual(int n, const int32_t* __restrict__ rp,
                                                               const int32_t* __restrict__ cols,
                                                               const double* __restrict__ vals,
                                                               const double* __restrict__ b,
                                                               const double* __restrict__ x,
                                                               const uint8_t* __restrict__ skip, double* partials,
                                                               unsigned int* ticket, double* out) {
  __shared__ double sh[kSolveBlock / 32];
  const int lane = threadIdx.x & (G - 1);
  const int groups = gridDim.x * (blockDim.x / G);
  const int nr = n + ((groups - n % groups) % groups);
  double rr = 0.0, bb = 0.0;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) / G; row < nr; row += groups) {
    double s = 0.0;
    if (row < n) s = row_dot<G>(row, rp, cols, vals, x, lane);
    else {
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
    }
    if (row < n && lane == 0 && !(skip && skip[row])) {
      double ri = b[row] - s;
      rr += ri * ri;
      bb += b[row] * b[row];
    }
  }
  rr = block_sum(rr, sh);
  bb = block_sum(bb, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x * 2] = rr;
    partials[blockIdx.x * 2 + 1] = bb;
  }
  if (last_block(ticket)) {
    double a = reduce_partials(partials, gridDim.x, 2, 0, sh);
    double c = reduce_partials(partials, gridDim.x, 2, 1, sh);
    if (threadIdx.x == 0) {
      out[0] = a;
      out[1] = c;
      *ticket = 0;
    }
  }
}

afem_status true_relres(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals,
                        int64_t nnz, const double* b, const double* x, const uint8_t* skip, double* relres) {
  const int G = lanes_per_row_fp64(n, nnz);
  const unsigned grid_rows = grid_for(ctx, (int64_t)n * G, kSolveBlock, 8);
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(double) * 2 * grid_rows) + 512));
  double *partials, *out;
  unsigned int* ticket;
  AFEM_TRY(scratch_take(ctx, 2 * (size_t)grid_rows, &partials));
  AFEM_TRY(scratch_take(ctx, 2, &out));
  AFEM_TRY(scratch_take(ctx, 1, &ticket));
  AFEM_CUDA(cudaMemsetAsync(ticket, 0, sizeof(unsigned int), ctx->stream));
  AFEM_TRY(dispatch_g(G, [&](auto g) {
    return launch(ctx, k_true_residual<decltype(g)::value>, grid_rows, kSolveBlock, 0, n, rp, cols, vals, b, x, skip,
                  partials, ticket, out);
  }));
  AFEM_CUDA(cudaMemcpyAsync(ctx->pinned, out, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
  const double* h = reinterpret_cast<const double*>(ctx->pinned);
  *relres = h[1] > 0 ? std::sqrt(h[0] / h[1]) : std::sqrt(h[0]);
  return AFEM_OK;
}

afem_status solve_csr(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals,
                      const double* b, double* x, const uint8_t* forced, const afem_solver_options* opt_in,
                      afem_solve_info* info) {
  AFEM_CHECK_ARG(ctx && n > 0 && rp && cols && vals && b && x, "afem_cg_solve_csr: bad arguments");
  afem_solver_options opt;
  if (opt_in) opt = *opt_in;
  else afem_solver_options_default(&opt);
  AFEM_CHECK_ARG(opt.precond == AFEM_PRECOND_NONE || opt.precond == AFEM_PRECOND_JACOBI,
                 "afem_cg_solve_csr: precond %d needs the learned-preconditioner entry points", opt.precond);
  int32_t nnz32 = 0;
  AFEM_TRY(read_scalar(ctx, rp + n, &nnz32));
  const int64_t nnz = nnz32;
  const uint8_t* skip = opt.skip_forced_rows ? forced : nullptr;
  cudaEvent_t e0, e1;
  AFEM_CUDA(cudaEventCreate(&e0));
  AFEM_CUDA(cudaEventCreate(&e1));
  AFEM_CUDA(cudaEventRecord(e0, ctx->stream));
  afem_status st = opt.precision == AFEM_PRECISION_MIXED ? cg_mixed(ctx, n, rp, cols, vals, nnz, b, x, skip, opt, info)
                                                         : cg_fp64(ctx, n, rp, cols, vals, nnz, b, x, skip, opt, info);
  cudaEventRecord(e1, ctx->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != AFEM_OK && st != AFEM_ERR_NOT_CONVERGED && st != AFEM_ERR_BREAKDOWN) return st;
  double rel = 0.0;
  afem_status s2 = true_relres(ctx, n, rp, cols, vals, nnz, b, x, skip, &rel);
  if (info) {
    info->solve_ms = ms;
    info->relres = rel;
    info->status = st;
  }
  if (s2 != AFEM_OK) return s2;
  if (st == AFEM_ERR_NOT_CONVERGED) return fail(st, "CG did not reach the tolerance (relres %.3e)", rel);
  if (st == AFEM_ERR_BREAKDOWN) return fail(st, "CG breakdown (<p, A p> <= 0 or non-finite)");
  return AFEM_OK;
}

afem_status spmv_fp64(afem_context ctx, int n, int64_t nnz, const int32_t* rp, const int32_t* cols,
                      const double* vals, const double* x, double* y) {
  const int G = lanes_per_row_fp64(n, nnz);
  const unsigned grid = grid_for(ctx, (int64_t)n * G, kSolveBlock, 8);
  return dispatch_g(G, [&](auto g) {
    return launch(ctx, k_spmv<decltype(g)::value>, grid, kSolveBlock, 0, n, rp, cols, vals, x, y);
  });
}

}  // namespace afem

using namespace afem;

extern "C" {

void afem_solver_options_default(afem_solver_options* o) {
  if (!o) return;
  o->rtol = 1e-7;
  o->atol = 0.0;
  o->max_iter = 1000;
  o->precond = AFEM_PRECOND_JACOBI;
  o->precision = AFEM_PRECISION_FP64;
  o->skip_forced_rows = 0;
  o->inner_rtol = 0.0;   // library default: 0.1
  o->check_every = 16;
  o->block_size = 0;
}

afem_status afem_cg_solve_csr(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals,
                              const double* b, double* x, const uint8_t* forced, const afem_solver_options* opt,
                              afem_solve_info* info) {
  return solve_csr(ctx, n, rp, cols, vals, b, x, forced, opt, info);
}

afem_status afem_spmv_csr(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals,
                          const double* x, double* y) {
  AFEM_CHECK_ARG(ctx && n > 0 && rp && cols && vals && x && y, "afem_spmv_csr: bad arguments");
  int32_t nnz = 0;
  AFEM_TRY(read_scalar(ctx, rp + n, &nnz));
  const int G = lanes_per_row_fp64(n, nnz);
  const unsigned grid = grid_for(ctx, (int64_t)n * G, kSolveBlock, 8);
  return dispatch_g(G, [&](auto g) {
    return launch(ctx, k_spmv<decltype(g)::value>, grid, kSolveBlock, 0, n, rp, cols, vals, x, y);
  });
}

}  // extern "C"
