// Factored sparse-approximate-inverse smoothers of the learned V-cycle.
//
// On the finest level and on every level of at most kFactRows rows above the
// level that is solved exactly, the V-cycle smooths with
//
//   G = theta L^T L,   L = (I + N) S,   S = diag(s),  s_i = sqrt(d_i),
//   L_ii = s_i,  L_ij = N_ij s_j = m_ij A_ij s_i s_j^2   (j < i, A_ij != 0),
//   m_ij = 2 tanh(ew . (o_i * o_j) + eb)                  (edge head on the level output o),
//   theta = kFactSafe / max(kFactSafe, max_i sum_j |(L^T L A)_ij|)
//
// in place of the weighted Jacobi step d * x.  L is lower triangular with a
// positive diagonal, so G is SPD, and the row-sum bound gives
// lambda_max(G A) < 2: the symmetric V-cycle stays SPD whatever the network
// outputs.  With zero edge heads, N = 0 and G = diag(d).
//
// L is stored as its strict lower part in row order (edge e = (i, j), j < i:
// lval[e], lo_col[e], rows by low_rp) plus the transposed index (the edges
// of column j: up_e[up_rp[j] .. up_rp[j+1]), rows lo_row[e]), and the diagonal
// sq.  The kernels of one vector take pointers already offset to it; the
// batched kernels take the vector from grid.y.
#pragma once

#include "afem_internal.cuh"
#include "afem_krylov.cuh"

namespace afem {

constexpr int kFactRows = 2048;      // levels of at most this many rows (and the finest) are factored
constexpr float kFactSafe = 1.9f;    // the row-sum bound of theta G A

struct FactView {
  int n = 0, nlow = 0;
  const int32_t *low_rp = nullptr, *lo_col = nullptr, *lo_row = nullptr, *up_rp = nullptr, *up_e = nullptr;
  const float *lval = nullptr, *sq = nullptr;
  const float* theta = nullptr;   // device scalar
};

// w = L x
__device__ __forceinline__ void fact_lower(int i0, int st, const FactView& f, const float* __restrict__ x,
                                           float* __restrict__ w) {
  for (int i = i0; i < f.n; i += st) {
    float acc = f.sq[i] * x[i];
    for (int32_t e = f.low_rp[i]; e < f.low_rp[i + 1]; ++e) acc = fmaf(f.lval[e], x[f.lo_col[e]], acc);
    w[i] = acc;
  }
}

// out = (base ? base : 0) + theta L^T (w1 + (w2 ? w2 : 0))
__device__ __forceinline__ void fact_upper(int i0, int st, const FactView& f, const float* __restrict__ w1,
                                           const float* __restrict__ w2, const float* __restrict__ base,
                                           float* __restrict__ out) {
  const float th = *f.theta;
  for (int j = i0; j < f.n; j += st) {
    float acc = f.sq[j] * (w2 ? w1[j] + w2[j] : w1[j]);
    for (int32_t k = f.up_rp[j]; k < f.up_rp[j + 1]; ++k) {
      const int32_t e = f.up_e[k], i = f.lo_row[e];
      acc = fmaf(f.lval[e], w2 ? w1[i] + w2[i] : w1[i], acc);
    }
    out[j] = base ? fmaf(th, acc, base[j]) : th * acc;
  }
}

// out = r - A x
__device__ __forceinline__ void vc_res(int i0, int st, int n, const int32_t* __restrict__ rp,
                                       const int32_t* __restrict__ cols, const float* __restrict__ w,
                                       const float* __restrict__ r, const float* __restrict__ x,
                                       float* __restrict__ out) {
  for (int i = i0; i < n; i += st) {
    float acc = r[i];
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) acc = fmaf(-w[k], x[cols[k]], acc);
    out[i] = acc;
  }
}

__global__ void k_fact_lower(FactView f, const float* __restrict__ x, float* __restrict__ w) {
  pdl_trigger();
  pdl_wait();
  const int64_t o = (int64_t)blockIdx.y * f.n;
  fact_lower(blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, f, x + o, w + o);
}

__global__ void k_fact_upper(FactView f, const float* __restrict__ w1, const float* __restrict__ w2,
                             const float* __restrict__ base, float* __restrict__ out) {
  pdl_trigger();
  pdl_wait();
  const int64_t o = (int64_t)blockIdx.y * f.n;
  fact_upper(blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, f, w1 + o, w2 ? w2 + o : nullptr,
             base ? base + o : nullptr, out + o);
}

__global__ void k_vc_res(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                         const float* __restrict__ w, const float* __restrict__ r, const float* __restrict__ x,
                         float* __restrict__ out) {
  pdl_trigger();
  pdl_wait();
  const int64_t o = (int64_t)blockIdx.y * n;
  vc_res(blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, n, rp, cols, w, r + o, x + o, out + o);
}

// ---------------------------------------------------------------------------
// Factor values from the network outputs (once per parameter set and operator).

// dst[e] = src[idx[e]]   (the lower entries' values of A_l)
__global__ void k_fact_gather(int n, const int32_t* __restrict__ idx, const float* __restrict__ src,
                              float* __restrict__ dst) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) dst[e] = src[idx[e]];
}

// s = sqrt(d)
__global__ void k_fact_sq(int n, const float* __restrict__ d, float* __restrict__ sq) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) sq[i] = sqrtf(d[i]);
}

// per edge: z = ew . (o_i * o_j) + eb, m = 2 tanh z, L_ij = m A_ij s_i s_j^2
__global__ void k_fact_edges(int nlow, const int32_t* __restrict__ lo_row, const int32_t* __restrict__ lo_col,
                             const float* __restrict__ a_low, const bf16* __restrict__ o, const float* __restrict__ ew,
                             const float* __restrict__ sq, float* __restrict__ z, float* __restrict__ m,
                             float* __restrict__ lval) {
  const float eb = ew[kF];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nlow; e += gridDim.x * blockDim.x) {
    const int32_t i = lo_row[e], j = lo_col[e];
    const __nv_bfloat162* oi = reinterpret_cast<const __nv_bfloat162*>(o + (int64_t)i * kF);
    const __nv_bfloat162* oj = reinterpret_cast<const __nv_bfloat162*>(o + (int64_t)j * kF);
    float acc = eb;
#pragma unroll 8
    for (int c = 0; c < kF / 2; ++c) {
      const float2 a = __bfloat1622float2(oi[c]), b = __bfloat1622float2(oj[c]);
      acc = fmaf(ew[2 * c] * a.x, b.x, acc);
      acc = fmaf(ew[2 * c + 1] * a.y, b.y, acc);
    }
    const float me = 2.f * tanhf(acc);
    const float sj = sq[j];
    z[e] = acc;
    m[e] = me;
    lval[e] = me * a_low[e] * sq[i] * sj * sj;
  }
}

// Per-thread accumulator table for one sparse row (columns -> values), in
// shared memory interleaved across the block's threads.
constexpr int kFactRowBlock = 32;
constexpr int kFactRowSlots = 128;   // distinct columns of a row of L^T L A (37 on a 7-point pattern)

__device__ __forceinline__ int fact_slot(int32_t j) { return (int)(((uint32_t)j * 2654435761u) >> 25); }

// Row sums of |L^T L A| (row i: sum over the column i of L, then the rows of
// L, then the rows of A), their maximum and the first row that attains it,
// packed as (float bits << 32 | ~row) for an atomicMax (row sums are >= 0).
// A row whose table fills sets the bound to +inf (theta = 0 is safe).
__global__ void __launch_bounds__(kFactRowBlock) k_fact_rows(FactView f, const int32_t* __restrict__ a_rp,
                                                             const int32_t* __restrict__ a_cols,
                                                             const float* __restrict__ a_w,
                                                             unsigned long long* __restrict__ packed) {
  __shared__ int32_t key[kFactRowSlots][kFactRowBlock];
  __shared__ float val[kFactRowSlots][kFactRowBlock];
  const int t = threadIdx.x;
  for (int h = 0; h < kFactRowSlots; ++h) key[h][t] = -1;
  unsigned long long best = 0;
  for (int i = blockIdx.x * blockDim.x + t; i < f.n; i += gridDim.x * blockDim.x) {
    bool full = false;
    // the column i of L: (k = i, L_ii) and (k = lo_row[e], L_ki) for the edges e of column i
    const int32_t kb = f.up_rp[i], ke = f.up_rp[i + 1];
    for (int32_t q = kb - 1; q < ke; ++q) {
      const int32_t k = q < kb ? i : f.lo_row[f.up_e[q]];
      const float lki = q < kb ? f.sq[i] : f.lval[f.up_e[q]];
      // the row k of L: (m = k, L_kk) and its lower edges
      for (int32_t p = f.low_rp[k] - 1; p < f.low_rp[k + 1]; ++p) {
        const int32_t mm = p < f.low_rp[k] ? k : f.lo_col[p];
        const float lkm = p < f.low_rp[k] ? f.sq[k] : f.lval[p];
        const float c = lki * lkm;
        for (int32_t a = a_rp[mm]; a < a_rp[mm + 1]; ++a) {
          const int32_t j = a_cols[a];
          int h = fact_slot(j);
          int probe = 0;
          for (; probe < kFactRowSlots; ++probe, h = (h + 1) & (kFactRowSlots - 1)) {
            const int32_t kk = key[h][t];
            if (kk == j) break;
            if (kk == -1) {
              key[h][t] = j;
              val[h][t] = 0.f;
              break;
            }
          }
          if (probe == kFactRowSlots) {
            full = true;
            continue;
          }
          val[h][t] = fmaf(c, a_w[a], val[h][t]);
        }
      }
    }
    float sum = 0.f;
    for (int h = 0; h < kFactRowSlots; ++h) {
      if (key[h][t] != -1) sum += fabsf(val[h][t]);
      key[h][t] = -1;
    }
    if (full) sum = __int_as_float(0x7f800000);   // +inf
    const unsigned long long pk = ((unsigned long long)__float_as_uint(sum) << 32) | (uint32_t)(~i);
    best = pk > best ? pk : best;
  }
  atomicMax(packed, best);
}

// theta = kFactSafe / max(kFactSafe, bound); bound and the row i* for the backward
__global__ void k_fact_theta(const unsigned long long* __restrict__ packed, float* __restrict__ theta,
                             float* __restrict__ bound, int* __restrict__ istar) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    const unsigned long long pk = *packed;
    const float b = __uint_as_float((uint32_t)(pk >> 32));
    *bound = b;
    *istar = (int)(~(uint32_t)pk);
    *theta = b > kFactSafe ? kFactSafe / b : 1.f;   // b = +inf gives 0
  }
}

// ---------------------------------------------------------------------------
// Backward.

// dL/dL on the diagonal and the lower edges of each row, and the partials of
// dL/dtheta, from the uses of G on the level: the pre-smoothing x1 = G r
// (wpre = L r, gpre = L x1b with x1b its adjoint) and the post-smoothing
// y = x2 + G u (wpost = L u, gpost = L g with g the adjoint of y; absent on
// the coarsest level).  For a use out = G a with adjoint gb:
//   dL/dL_ij += theta ((L gb)_i a_j + (L a)_i gb_j),  dL/dtheta += (L gb) . (L a).
__global__ void k_fact_grad(FactView f, int batch, const float* __restrict__ r, const float* __restrict__ x1b,
                            const float* __restrict__ wpre, const float* __restrict__ gpre,
                            const float* __restrict__ u, const float* __restrict__ g,
                            const float* __restrict__ wpost, const float* __restrict__ gpost,
                            float* __restrict__ gl_diag, float* __restrict__ gl_low, float* __restrict__ dth_part) {
  __shared__ double sh[32];
  const float th = *f.theta;
  float dth = 0.f;
  const int n = f.n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float gd = 0.f;
    for (int b = 0; b < batch; ++b) {
      const int64_t k = (int64_t)b * n + i;
      gd = fmaf(gpre[k], r[k], fmaf(wpre[k], x1b[k], gd));
      dth = fmaf(gpre[k], wpre[k], dth);
      if (u) {
        gd = fmaf(gpost[k], u[k], fmaf(wpost[k], g[k], gd));
        dth = fmaf(gpost[k], wpost[k], dth);
      }
    }
    gl_diag[i] = th * gd;
    for (int32_t e = f.low_rp[i]; e < f.low_rp[i + 1]; ++e) {
      const int32_t j = f.lo_col[e];
      float ge = 0.f;
      for (int b = 0; b < batch; ++b) {
        const int64_t ki = (int64_t)b * n + i, kj = (int64_t)b * n + j;
        ge = fmaf(gpre[ki], r[kj], fmaf(wpre[ki], x1b[kj], ge));
        if (u) ge = fmaf(gpost[ki], u[kj], fmaf(wpost[ki], g[kj], ge));
      }
      gl_low[e] = th * ge;
    }
  }
  const double tot = block_sum((double)dth, sh);
  if (threadIdx.x == 0) dth_part[blockIdx.x] = (float)tot;
}

// theta = kFactSafe / bound when bound > kFactSafe: dL/dL += dL/dtheta dtheta/dbound dbound/dL through the row i*
// that attains the bound,
//   bound = sum_j sigma_j sum_k L_{k i*} sum_m L_km A_mj  (sigma_j the sign of (L^T L A)_{i* j}),
//   dbound/dL_{k i*} = (L A sigma)_k,  dbound/dL_km += L_{k i*} (A sigma)_m.
// One thread; the signs come from the same accumulation as k_fact_rows.
__global__ void k_fact_theta_grad(FactView f, const int32_t* __restrict__ a_rp, const int32_t* __restrict__ a_cols,
                                  const float* __restrict__ a_w, const float* __restrict__ bound_d,
                                  const int* __restrict__ istar_d, const float* __restrict__ dth,
                                  float* __restrict__ gl_diag, float* __restrict__ gl_low) {
  __shared__ int32_t key[kFactRowSlots];
  __shared__ float val[kFactRowSlots];
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const float bound = *bound_d;
  if (!(bound > kFactSafe) || !(bound < __int_as_float(0x7f800000))) return;
  const float db = *dth * (-kFactSafe / (bound * bound));
  const int32_t is = *istar_d;
  for (int h = 0; h < kFactRowSlots; ++h) key[h] = -1;
  auto slot = [&](int32_t j, bool insert) {
    int h = fact_slot(j);
    for (int p = 0; p < kFactRowSlots; ++p, h = (h + 1) & (kFactRowSlots - 1)) {
      if (key[h] == j) return h;
      if (key[h] == -1) {
        if (!insert) return -1;
        key[h] = j;
        val[h] = 0.f;
        return h;
      }
    }
    return -1;
  };
  const int32_t kb = f.up_rp[is], ke = f.up_rp[is + 1];
  for (int pass = 0; pass < 2; ++pass) {
    for (int32_t q = kb - 1; q < ke; ++q) {
      const int32_t k = q < kb ? is : f.lo_row[f.up_e[q]];
      const float lki = q < kb ? f.sq[is] : f.lval[f.up_e[q]];
      float las = 0.f;   // (L A sigma)_k
      for (int32_t p = f.low_rp[k] - 1; p < f.low_rp[k + 1]; ++p) {
        const int32_t mm = p < f.low_rp[k] ? k : f.lo_col[p];
        const float lkm = p < f.low_rp[k] ? f.sq[k] : f.lval[p];
        float as = 0.f;   // (A sigma)_m
        for (int32_t a = a_rp[mm]; a < a_rp[mm + 1]; ++a) {
          const int32_t j = a_cols[a];
          const int h = slot(j, pass == 0);
          if (h < 0) continue;
          if (pass == 0) {
            val[h] = fmaf(lki * lkm, a_w[a], val[h]);
          } else {
            const float sg = val[h] > 0.f ? 1.f : (val[h] < 0.f ? -1.f : 0.f);
            as = fmaf(a_w[a], sg, as);
          }
        }
        if (pass == 1) {
          las = fmaf(lkm, as, las);
          // dbound/dL_km += L_{k i*} (A sigma)_m
          if (p < f.low_rp[k]) gl_diag[k] += db * lki * as;
          else gl_low[p] += db * lki * as;
        }
      }
      // dbound/dL_{k i*} += (L A sigma)_k
      if (pass == 1) {
        if (q < kb) gl_diag[is] += db * las;
        else gl_low[f.up_e[q]] += db * las;
      }
    }
  }
}

// dL/dc of a factored level: through L_ii = s_i and L_ij = m A_ij s_i s_j^2 to
// ds, dd = ds / (2 s), then d = cap sigmoid(c + logit 0.8) as the diagonal levels
__global__ void k_fact_dc(FactView f, const float* __restrict__ m, const float* __restrict__ a_low,
                          const float* __restrict__ gl_diag, const float* __restrict__ gl_low,
                          const float* __restrict__ d, const float* __restrict__ cap, float* __restrict__ dc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < f.n; i += gridDim.x * blockDim.x) {
    const float si = f.sq[i];
    float ds = gl_diag[i];
    for (int32_t e = f.low_rp[i]; e < f.low_rp[i + 1]; ++e) {
      const float sj = f.sq[f.lo_col[e]];
      ds = fmaf(gl_low[e] * m[e] * a_low[e], sj * sj, ds);
    }
    for (int32_t k = f.up_rp[i]; k < f.up_rp[i + 1]; ++k) {
      const int32_t e = f.up_e[k];
      ds = fmaf(gl_low[e] * m[e] * a_low[e], 2.f * f.sq[f.lo_row[e]] * si, ds);
    }
    const float di = d[i], ci = cap[i];
    const float dd = si > 0.f ? ds / (2.f * si) : 0.f;
    dc[i] = ci > 0.f ? dd * di * (1.f - di / ci) : 0.f;
  }
}

// dz_e = dL/dL_ij A_ij s_i s_j^2 2 (1 - tanh^2 z), and per-block partials of
// the edge head's gradient: dew = sum_e dz_e (o_i * o_j), deb = sum_e dz_e
__global__ void k_fact_edge_backward(FactView f, const float* __restrict__ z, const float* __restrict__ a_low,
                                     const float* __restrict__ gl_low, const bf16* __restrict__ o,
                                     float* __restrict__ dz, float* __restrict__ part) {
  __shared__ float sh[kF + 1][8];
  float acc[kF + 1];
#pragma unroll
  for (int c = 0; c <= kF; ++c) acc[c] = 0.f;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < f.nlow; e += gridDim.x * blockDim.x) {
    const int32_t i = f.lo_row[e], j = f.lo_col[e];
    const float th = tanhf(z[e]);
    const float sj = f.sq[j];
    const float g = gl_low[e] * a_low[e] * f.sq[i] * sj * sj * 2.f * (1.f - th * th);
    dz[e] = g;
    const __nv_bfloat162* oi = reinterpret_cast<const __nv_bfloat162*>(o + (int64_t)i * kF);
    const __nv_bfloat162* oj = reinterpret_cast<const __nv_bfloat162*>(o + (int64_t)j * kF);
#pragma unroll
    for (int c = 0; c < kF / 2; ++c) {
      const float2 a = __bfloat1622float2(oi[c]), b = __bfloat1622float2(oj[c]);
      acc[2 * c] = fmaf(g * a.x, b.x, acc[2 * c]);
      acc[2 * c + 1] = fmaf(g * a.y, b.y, acc[2 * c + 1]);
    }
    acc[kF] += g;
  }
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c <= kF; ++c) {
    float v = acc[c];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    if (lane == 0) sh[c][wp] = v;
  }
  __syncthreads();
  if (threadIdx.x <= kF) {
    float s = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[threadIdx.x][k];
    part[(int64_t)blockIdx.x * (kF + 1) + threadIdx.x] = s;
  }
}

// dO_i += sum over the edges e of node i (as row and as column) of dz_e ew * o_other; one warp per node,
// two features per lane
__global__ void k_fact_dO(FactView f, const float* __restrict__ dz, const bf16* __restrict__ o,
                          const float* __restrict__ ew, float* __restrict__ dO) {
  const int lane = threadIdx.x & 31;
  const float w0 = ew[2 * lane], w1 = ew[2 * lane + 1];
  for (int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; i < f.n;
       i += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    float a0 = 0.f, a1 = 0.f;
    for (int32_t e = f.low_rp[i]; e < f.low_rp[i + 1]; ++e) {
      const float2 v = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(o + (int64_t)f.lo_col[e] * kF)[lane]);
      a0 = fmaf(dz[e], v.x, a0);
      a1 = fmaf(dz[e], v.y, a1);
    }
    for (int32_t k = f.up_rp[i]; k < f.up_rp[i + 1]; ++k) {
      const int32_t e = f.up_e[k];
      const float2 v = __bfloat1622float2(reinterpret_cast<const __nv_bfloat162*>(o + (int64_t)f.lo_row[e] * kF)[lane]);
      a0 = fmaf(dz[e], v.x, a0);
      a1 = fmaf(dz[e], v.y, a1);
    }
    float2* drow = reinterpret_cast<float2*>(dO + i * kF);
    const float2 cur = drow[lane];
    drow[lane] = make_float2(fmaf(w0, a0, cur.x), fmaf(w1, a1, cur.y));
  }
}

}  // namespace afem
