// Learned preconditioner: a geometric multigrid V-cycle whose per-node
// smoother weights are predicted by a message-passing network (MPNN) on the
// mesh graph, trained on the GPU and applied inside flexible CG.
//
// Preconditioner: one symmetric V(1,1)-cycle from a zero initial guess on the
// Galerkin hierarchy A_0 = A, A_{l+1} = P_l^T A_l P_l (P_l the caller's
// prolongation, computed here in FP64 on the caller's coarse patterns):
//   V_l(r):  x1 = d_l .* r ;  s = r - A_l x1
//            x2 = x1 + P_l V_{l+1}(P_l^T s)
//            u  = r - A_l x2 ;  return x2 + d_l .* u
//   V_{L-1}(r) = d_{L-1} .* r
// Weighted-Jacobi smoothers with per-node weights
//   d_l = cap_l * sigmoid(c_l + logit(0.8)),  cap_l = 2 / sum_j |A_l,ij|
// (0 on empty rows): 2 diag(d_l)^-1 - A_l is strictly diagonally dominant, so
// the V-cycle is symmetric positive definite whatever the network predicts;
// c = 0 is l1-Jacobi smoothing at 0.8 of the cap.  The caller's P_l should
// vanish on Dirichlet nodes (rows of fine and columns of coarse boundary
// nodes), so that the coarse spaces satisfy the boundary condition.
// Fine levels run one kernel per step; the levels of <= kCoarseRows rows run
// in ONE block per vector with block barriers.
//
// Network (message-passing layers of width 64, BF16 weights and activations,
// FP32 accumulation) on the coefficient features x0 = [1, log(A_ii / mean)]:
//   a = relu(x0 W_in + b_in)
//   o_l = relu(h_l W1_l + (S_l h_l) W2_l + b_l),  h_0 = a,  h_{l+1} = R_l o_l
//   (levels past the last layer: o_l = h_l)
//   c_l = o_l . w_l + beta_l                      (one head per level)
// S_0 is the matrix graph with weights -A_ij / sqrt(A_ii A_jj); S_l (l >= 1),
// R_l, P_l come from the caller (CSR).  It runs once per operator and per
// training step; the per-iteration application is the V-cycle above.
//
// GEMMs on the 5th-generation tensor cores (tcgen05.mma, BF16 -> FP32 in
// TMEM, operand tiles by TMA): the row GEMMs of the forward pass and of the
// backward dX (K = 64), and the weight gradients X^T G (64 x 64 results
// summed over all rows, MN-major operands).  Aggregation / transfers: CSR
// SpMM over 64-wide rows.  Training: the mean relative energy norm of the
// error propagation, ||(I - M A) e||_A^2 / ||e||_A^2 over (r = A e, e) pairs
// (A in FP32), back-propagated through the adjoint V-cycle; Adam on FP32
// master weights.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "afem_krylov.cuh"

namespace afem {

constexpr int kF = 64;                 // hidden width
constexpr int kMaxLevels = 12;
constexpr int kMaxBatch = 64;
constexpr float kLogitTheta = 1.38629436f;   // log(0.8 / 0.2): untrained weight = 0.8 of the l1 cap

typedef __nv_bfloat16 bf16;

// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

// ---------------------------------------------------------------------------
// Row GEMM on the 5th-generation tensor cores:
//   Y[M x 64] = act( X1 B1 + X2 B2 + bias ),  X in BF16 (row-major, 64 columns),
// B given transposed as Bt[n][k] (64 x 64 BF16, i.e. K-major), FP32 accumulate;
// output BF16 (Yb) and/or FP32 (Yf, optionally accumulated).
//
// Persistent CTAs of 128 threads walk 128-row tiles.  Bt1/Bt2 are staged once
// into shared memory in the 128-byte-swizzled K-major layout (16-byte chunk c
// of row r at r * 128 + ((c ^ (r & 7)) << 4), tile base 1024-byte aligned).
// The X tiles arrive by TMA (cp.async.bulk.tensor.2d, SWIZZLE_128B, the same
// layout; rows past M read as zero) into a two-stage ring completed on an
// mbarrier transaction count: the next tile's copy is in flight while the
// current tile is multiplied and written out.  Thread 0 issues the
// tcgen05.mma (M = 128, N = 64, K = 16; 4 per product) into a 64-column TMEM
// accumulator and commits them to a second mbarrier; warp w then reads TMEM
// lanes 32 w .. 32 w + 31 (its tile rows) with tcgen05.ld and applies bias,
// ReLU and the stores.  Every mbarrier wait is bounded: on timeout the kernel
// sets *err, waits (bounded) for its own copy in flight, frees its TMEM and
// returns.
constexpr int kTcRows = 128;                 // rows per tile (MMA M)
constexpr int kTcTileBytes = kTcRows * 128;  // one BF16 X tile
constexpr long long kTcWaitCycles = 2000000000ll;
// kind::f16 instruction descriptor: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit 17,
// M >> 4 at bit 24.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kF >> 3) << 17) |
                              ((uint32_t)(kTcRows >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, 128-byte swizzle, K-major: start address
// >> 4 (bits 0-13), leading byte offset 16 B (unused for this layout), stride
// byte offset 1024 B between 8-row groups (bits 32-45), descriptor version 1
// (bits 46-47), layout SWIZZLE_128B = 2 (bits 61-63).  K steps of 16 elements
// advance the start address by 32 B inside the swizzle atom.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)1 << 16) | ((uint64_t)(1024 >> 4) << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

// bounded wait for phase `parity` of an mbarrier; false on timeout
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  for (;;) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > kTcWaitCycles) return false;
  }
}

template <bool TWO>
__device__ __forceinline__ void tc_load_tile(uint32_t bar, uint32_t dst1, const CUtensorMap* m1, uint32_t dst2,
                                             const CUtensorMap* m2, int row) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
               "r"((uint32_t)(TWO ? 2 : 1) * kTcTileBytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst1),
      "l"(reinterpret_cast<uint64_t>(m1)), "r"(0), "r"(row), "r"(bar)
      : "memory");
  if (TWO)
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            dst2),
        "l"(reinterpret_cast<uint64_t>(m2)), "r"(0), "r"(row), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tc_stage_weights(const bf16* __restrict__ Bt, uint8_t* sB) {
  for (int e = threadIdx.x; e < kF * 8; e += blockDim.x) {
    const int r = e >> 3, c = e & 7;
    const uint4 v = *reinterpret_cast<const uint4*>(Bt + r * kF + c * 8);
    *reinterpret_cast<uint4*>(sB + r * 128 + ((c ^ (r & 7)) << 4)) = v;
  }
}

template <bool TWO>
constexpr int tc_smem_bytes() {
  // weights, two X stages, barriers + TMEM slot, bias; plus 1024 for the alignment of the base
  return (TWO ? 2 : 1) * kF * 128 + 2 * (TWO ? 2 : 1) * kTcTileBytes + 64 + kF * 4 + 1024;
}

template <bool TWO, bool RELU>
__global__ void __launch_bounds__(128) k_row_gemm(const __grid_constant__ CUtensorMap mX1,
                                                  const __grid_constant__ CUtensorMap mX2, int M,
                                                  const bf16* __restrict__ B1t, const bf16* __restrict__ B2t,
                                                  const float* __restrict__ bias, bf16* __restrict__ Yb,
                                                  float* __restrict__ Yf, int accumulate, int* __restrict__ err) {
  extern __shared__ uint8_t tc_dyn[];
  uint8_t* const base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_dyn) + 1023) & ~(uintptr_t)1023);
  constexpr int NP = TWO ? 2 : 1;
  uint8_t* const sB = base;                                   // NP x 8 KB
  uint8_t* const sX = base + NP * kF * 128;                   // [stage][product] 16 KB tiles
  uint64_t* const bars = reinterpret_cast<uint64_t*>(sX + 2 * NP * kTcTileBytes);   // full[2], mma
  uint32_t* const tslot = reinterpret_cast<uint32_t*>(bars + 3);
  float* const sbias = reinterpret_cast<float*>(bars + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntiles = (M + kTcRows - 1) / kTcRows;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int b = 0; b < 3; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bars + b)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_stage_weights(B1t, sB);
  if (TWO) tc_stage_weights(B2t, sB + kF * 128);
  if (tid < kF) sbias[tid] = bias ? bias[tid] : 0.f;
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t full0 = smem_u32(bars), mma_bar = smem_u32(bars + 2);
  auto stage_x = [&](int st, int p) { return smem_u32(sX + (st * NP + p) * kTcTileBytes); };

  // per stage (thread 0): a copy issued and not yet waited for, and the completed waits (phase parity)
  bool outstanding[2] = {false, false};
  uint32_t uses[2] = {0u, 0u};
  if (tid == 0 && (int)blockIdx.x < ntiles) {
    tc_load_tile<TWO>(full0, stage_x(0, 0), &mX1, stage_x(0, 1), &mX2, blockIdx.x * kTcRows);
    outstanding[0] = true;
  }
  bool failed = false;
  int it = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
    const int st = it & 1;
    bool ok = true;
    if (tid == 0) {
      const int next = tile + gridDim.x;
      // stage st ^ 1 was last read by the previous tile's MMAs, complete before the barrier that ended it
      if (next < ntiles) {
        tc_load_tile<TWO>(full0 + 8 * (st ^ 1), stage_x(st ^ 1, 0), &mX1, stage_x(st ^ 1, 1), &mX2, next * kTcRows);
        outstanding[st ^ 1] = true;
      }
      ok = mbar_wait(full0 + 8 * st, uses[st] & 1u);
      if (ok) {
        ++uses[st];
        outstanding[st] = false;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int p = 0; p < NP; ++p)
#pragma unroll
          for (int kk = 0; kk < kF / 16; ++kk) {
            const uint64_t ad = sw128_desc(stage_x(st, p) + 32 * kk);
            const uint64_t bd = sw128_desc(smem_u32(sB + p * kF * 128) + 32 * kk);
            const uint32_t acc = (p | kk) != 0;
            asm volatile(
                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
                "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(acc)
                : "memory");
          }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mma_bar)
                     : "memory");
      }
    }
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    ok = __all_sync(0xffffffffu, mbar_wait(mma_bar, it & 1));
    if (__syncthreads_or(!ok)) {
      failed = true;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    float v[kF];
#pragma unroll
    for (int q = 0; q < kF / 16; ++q) {
      uint32_t r[16];
      const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + 16 * q;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
      for (int j = 0; j < 16; ++j) v[16 * q + j] = __uint_as_float(r[j]) + sbias[16 * q + j];
    }
    const int64_t row = (int64_t)tile * kTcRows + 32 * warp + lane;
    if (row < M) {
      if (RELU)
#pragma unroll
        for (int j = 0; j < kF; ++j) v[j] = fmaxf(v[j], 0.f);
      if (Yb) {
        uint4* dst = reinterpret_cast<uint4*>(Yb + row * kF);
#pragma unroll
        for (int c = 0; c < kF / 8; ++c)
          dst[c] = make_uint4(pack_bf16(v[8 * c], v[8 * c + 1]), pack_bf16(v[8 * c + 2], v[8 * c + 3]),
                              pack_bf16(v[8 * c + 4], v[8 * c + 5]), pack_bf16(v[8 * c + 6], v[8 * c + 7]));
      }
      if (Yf) {
        float4* dst = reinterpret_cast<float4*>(Yf + row * kF);
#pragma unroll
        for (int c = 0; c < kF / 4; ++c) {
          float4 o = accumulate ? dst[c] : make_float4(0.f, 0.f, 0.f, 0.f);
          dst[c] = make_float4(o.x + v[4 * c], o.y + v[4 * c + 1], o.z + v[4 * c + 2], o.w + v[4 * c + 3]);
        }
      }
    }
    // TMEM is overwritten by the next tile's MMAs only after every warp has read it
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  if (failed) {
    if (tid == 0) {
      atomicExch(err, 1);
      for (int b = 0; b < 2; ++b)   // our own copies still in flight
        if (outstanding[b]) (void)mbar_wait(full0 + 8 * b, uses[b] & 1u);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  }
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem));
}

// Weight-gradient partials on the tensor cores: per CTA
//   P[128 x 64] = [X1^T ; X2^T] G   summed over its 128-row tiles,
// X1, X2, G BF16 [M x 64] row-major (P rows 0..63: X1^T G, rows 64..127: X2^T G,
// FP32 out at partial[blockIdx.x]).  The reduction runs over rows, so both
// operands are MN-major: a 128-row TMA tile with the 128-byte swizzle is one
// MN-major swizzle atom (64 elements along M or N, 8-row K groups 1024 B
// apart), and A stacks the X1 and X2 tiles as two atoms along M (leading byte
// offset = one tile).  Each K step of 16 rows advances the start addresses by
// 2048 B.  A two-stage TMA ring (full / empty mbarriers): the next tile's
// copy runs while the current tile is multiplied, and a stage is refilled
// once the MMAs that read it have committed.  The accumulator stays in TMEM
// across the CTA's tiles; bounded waits as in k_row_gemm.
constexpr int kDwSmem = 2 * 3 * kTcTileBytes + 64 + 1024;
// kind::f16, D FP32, A and B BF16 and MN-major (bits 15, 16), N = 64, M = 128
constexpr uint32_t kDwIdesc = kTcIdesc | (1u << 15) | (1u << 16);

__device__ __forceinline__ uint64_t mn128_desc(uint32_t addr, uint32_t atom_stride) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((atom_stride >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)(1024 >> 4) << 32) | ((uint64_t)1 << 46) | ((uint64_t)2 << 61);
}

__global__ void __launch_bounds__(128) k_dw_grad(const __grid_constant__ CUtensorMap mX1,
                                                 const __grid_constant__ CUtensorMap mX2,
                                                 const __grid_constant__ CUtensorMap mG, int M,
                                                 float* __restrict__ partial, int* __restrict__ err) {
  extern __shared__ uint8_t tc_dyn[];
  uint8_t* const base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_dyn) + 1023) & ~(uintptr_t)1023);
  // stage s: X1 tile, X2 tile (the two A atoms, adjacent), G tile
  uint64_t* const bars = reinterpret_cast<uint64_t*>(base + 2 * 3 * kTcTileBytes);   // full[2], empty[2]
  uint32_t* const tslot = reinterpret_cast<uint32_t*>(bars + 4);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ntiles = (M + kTcRows - 1) / kTcRows;
  const int nlocal = (ntiles - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;   // >= 1 (grid <= ntiles)
  auto tile_at = [&](int st, int p) { return smem_u32(base + (st * 3 + p) * kTcTileBytes); };

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    for (int b = 0; b < 4; ++b) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bars + b)));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tslot;
  const uint32_t full0 = smem_u32(bars), empty0 = smem_u32(bars + 2);

  bool ok = true;
  if (tid == 0) {
    bool loaded[2] = {false, false}, committed[2] = {false, false};
    uint32_t full_uses[2] = {0u, 0u}, empty_uses[2] = {0u, 0u};
    auto load = [&](int st, int local) {
      const int row = (blockIdx.x + local * gridDim.x) * kTcRows;
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(full0 + 8 * st),
                   "r"((uint32_t)3 * kTcTileBytes)
                   : "memory");
      const CUtensorMap* maps[3] = {&mX1, &mX2, &mG};
#pragma unroll
      for (int p = 0; p < 3; ++p)
        asm volatile(
            "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
                "r"(tile_at(st, p)),
            "l"(reinterpret_cast<uint64_t>(maps[p])), "r"(0), "r"(row), "r"(full0 + 8 * st)
            : "memory");
      loaded[st] = true;
    };
    load(0, 0);
    for (int it = 0; it < nlocal && ok; ++it) {
      const int st = it & 1;
      if (it + 1 < nlocal) {   // refill the other stage once the MMAs of tile it - 1 are done with it
        if (committed[st ^ 1]) {
          ok = mbar_wait(empty0 + 8 * (st ^ 1), empty_uses[st ^ 1] & 1u);
          if (!ok) break;
          ++empty_uses[st ^ 1];
          committed[st ^ 1] = false;
        }
        load(st ^ 1, it + 1);
      }
      ok = mbar_wait(full0 + 8 * st, full_uses[st] & 1u);
      if (!ok) break;
      ++full_uses[st];
      loaded[st] = false;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
      for (int kk = 0; kk < kTcRows / 16; ++kk) {
        const uint64_t ad = mn128_desc(tile_at(st, 0) + 2048 * kk, kTcTileBytes);
        const uint64_t bd = mn128_desc(tile_at(st, 2) + 2048 * kk, 1024);   // one atom along N
        const uint32_t acc = (it | kk) != 0;
        asm volatile(
            "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(kDwIdesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(empty0 + 8 * st)
                   : "memory");
      committed[st] = true;
    }
    // the last MMAs (and, after a failure, our own copies in flight)
    for (int b = 0; b < 2; ++b) {
      if (committed[b]) ok = mbar_wait(empty0 + 8 * b, empty_uses[b] & 1u) && ok;
      if (loaded[b]) (void)mbar_wait(full0 + 8 * b, full_uses[b] & 1u);
    }
    if (!ok) atomicExch(err, 1);
  }
  ok = __syncthreads_and(tid == 0 ? ok : 1);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (ok) {
    float* out = partial + (int64_t)blockIdx.x * 2 * kF * kF + (32 * warp + lane) * kF;
#pragma unroll
    for (int q = 0; q < kF / 16; ++q) {
      uint32_t r[16];
      const uint32_t ta = tmem + ((uint32_t)(32 * warp) << 16) + 16 * q;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(ta));
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      float4* o4 = reinterpret_cast<float4*>(out + 16 * q);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        o4[j] = make_float4(__uint_as_float(r[4 * j]), __uint_as_float(r[4 * j + 1]), __uint_as_float(r[4 * j + 2]),
                            __uint_as_float(r[4 * j + 3]));
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem));
}

// out[e] (+)= sum_b partial[b][e] in a fixed order (deterministic).  A block
// covers 32 consecutive elements, one per lane, so that every warp load is
// one coalesced 128-byte row segment; its kSumWarps warps split the partials
// (warp w takes b = w, w + kSumWarps, ..., four loads in flight), and warp 0
// adds the warp sums in warp order.
constexpr int kSumWarps = 32;
__global__ void __launch_bounds__(32 * kSumWarps) k_sum_partials(int nparts, int nelem,
                                                                 const float* __restrict__ partial,
                                                                 float* __restrict__ out, int accumulate) {
  __shared__ float sh[kSumWarps][33];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int e = blockIdx.x * 32 + lane;
  float s = 0.f;
  if (e < nelem) {
    int b = w;
    for (; b + 3 * kSumWarps < nparts; b += 4 * kSumWarps) {
      const float a0 = partial[(int64_t)b * nelem + e];
      const float a1 = partial[(int64_t)(b + kSumWarps) * nelem + e];
      const float a2 = partial[(int64_t)(b + 2 * kSumWarps) * nelem + e];
      const float a3 = partial[(int64_t)(b + 3 * kSumWarps) * nelem + e];
      s += a0;
      s += a1;
      s += a2;
      s += a3;
    }
    for (; b < nparts; b += kSumWarps) s += partial[(int64_t)b * nelem + e];
  }
  sh[w][lane] = s;
  __syncthreads();
  if (w == 0 && e < nelem) {
    float t = 0.f;
    for (int k = 0; k < kSumWarps; ++k) t += sh[k][lane];
    out[e] = accumulate ? out[e] + t : t;
  }
}

// ---------------------------------------------------------------------------
// CSR SpMM over 64-wide rows, one warp per row, lane = 2 features.
// Y[b][row] = (acc ? Y : 0) + sum_k w_k X[b][col_k] (+ Z[b][row])  ; batch in grid.y.
template <class TIn, class TOut>
__global__ void k_spmm(int nrow, int ncol_rows, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                       const float* __restrict__ w, const TIn* __restrict__ X, const bf16* __restrict__ Z,
                       TOut* __restrict__ Y, int accumulate) {
  const int lane = threadIdx.x & 31;
  const int64_t b = blockIdx.y;
  const TIn* Xb = X + b * (int64_t)ncol_rows * kF;
  TOut* Yb = Y + b * (int64_t)nrow * kF;
  const bf16* Zb = Z ? Z + b * (int64_t)nrow * kF : nullptr;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; row < nrow; row += (gridDim.x * blockDim.x) >> 5) {
    float s0 = 0.f, s1 = 0.f;
    for (int32_t k = rp[row]; k < rp[row + 1]; ++k) {
      const float wk = w[k];
      const int64_t c = cols[k];
      float x0, x1;
      if constexpr (sizeof(TIn) == 2) {
        const __nv_bfloat162 v = reinterpret_cast<const __nv_bfloat162*>(Xb + c * kF)[lane];
        x0 = __low2float(v);
        x1 = __high2float(v);
      } else {
        const float2 v = reinterpret_cast<const float2*>(Xb + c * kF)[lane];
        x0 = v.x;
        x1 = v.y;
      }
      s0 = fmaf(wk, x0, s0);
      s1 = fmaf(wk, x1, s1);
    }
    if (Zb) {
      const __nv_bfloat162 z = reinterpret_cast<const __nv_bfloat162*>(Zb + (int64_t)row * kF)[lane];
      s0 += __low2float(z);
      s1 += __high2float(z);
    }
    if constexpr (sizeof(TOut) == 2) {
      reinterpret_cast<__nv_bfloat162*>(Yb + (int64_t)row * kF)[lane] = __floats2bfloat162_rn(s0, s1);
    } else {
      float2* p = reinterpret_cast<float2*>(Yb + (int64_t)row * kF) + lane;
      float2 o = accumulate ? *p : make_float2(0.f, 0.f);
      *p = make_float2(o.x + s0, o.y + s1);
    }
  }
}

// ---------------------------------------------------------------------------
// Small per-node kernels.

// Level-0 graph weights from A: w_ij = -A_ij / sqrt(A_ii A_jj), 0 on the diagonal.
__global__ void k_level0_weights(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                                 const double* __restrict__ vals, const double* __restrict__ diag,
                                 float* __restrict__ w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double di = diag[i];
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
      const int32_t j = cols[k];
      w[k] = (j == i) ? 0.f : (float)(-vals[k] / sqrt(di * diag[j]));
    }
  }
}

__global__ void k_diag(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                       const double* __restrict__ vals, double* __restrict__ diag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double d = 1.0;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
      if (cols[k] == i) {
        d = vals[k];
        break;
      }
    d = d > 0 ? d : 1.0;
    diag[i] = d;
  }
}

// coefficient features x0 = [1, log d - mean log d] and the input layer a = relu(x0 W_in + b_in)
__global__ void k_input_layer(int n, const double* __restrict__ diag, double mean_log, const float* __restrict__ Win,
                              const float* __restrict__ bin, float* __restrict__ x0, bf16* __restrict__ a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float f0 = 1.f;
    const float f1 = (float)(log(diag[i]) - mean_log);
    x0[2 * (int64_t)i] = f0;
    x0[2 * (int64_t)i + 1] = f1;
    __nv_bfloat162* dst = reinterpret_cast<__nv_bfloat162*>(a + (int64_t)i * kF);
#pragma unroll 8
    for (int c = 0; c < kF; c += 2) {
      const float y0 = fmaxf(f0 * Win[c] + f1 * Win[kF + c] + bin[c], 0.f);
      const float y1 = fmaxf(f0 * Win[c + 1] + f1 * Win[kF + c + 1] + bin[c + 1], 0.f);
      dst[c / 2] = __floats2bfloat162_rn(y0, y1);
    }
  }
}

// level head: c = o . w + beta ; d = cap * sigmoid(clamp(c + logit(0.8)))
__global__ void k_head(int n, const bf16* __restrict__ o, const float* __restrict__ w, const float* __restrict__ base,
                       float* __restrict__ d) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const __nv_bfloat162* row = reinterpret_cast<const __nv_bfloat162*>(o + (int64_t)i * kF);
    float acc = w[kF];
#pragma unroll 8
    for (int c = 0; c < kF / 2; ++c) {
      const __nv_bfloat162 v = row[c];
      acc = fmaf(__low2float(v), w[2 * c], acc);
      acc = fmaf(__high2float(v), w[2 * c + 1], acc);
    }
    d[i] = base[i] / (1.f + __expf(-fminf(fmaxf(acc + kLogitTheta, -30.f), 30.f)));
  }
}

// scalar CSR SpMV over a batch (grid.y): y[b][i] = (d ? d[i] t[b][i] : 0) + sum_k w_k x[b][col_k]
__global__ void k_sweep(int nrow, int ncol, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                        const float* __restrict__ w, const float* __restrict__ x, const float* __restrict__ d,
                        const float* __restrict__ t, const float* __restrict__ add, float* __restrict__ y) {
  pdl_trigger();
  pdl_wait();
  const int64_t b = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nrow; i += gridDim.x * blockDim.x) {
    float s = d ? d[i] * t[b * nrow + i] : (add ? add[b * nrow + i] : 0.f);
    if (x)
      for (int32_t k = rp[i]; k < rp[i + 1]; ++k) s = fmaf(w[k], x[b * ncol + cols[k]], s);
    y[b * nrow + i] = s;
  }
}

// ---------------------------------------------------------------------------
// V-cycle kernels (FP32).  The row operations below are shared by the
// per-level kernels (grid-stride over the rows of one vector, the vector in
// grid.y) and the coarse-levels kernels (block-stride, one block per vector).
// Pointers are already offset to the vector.

// s = r - A (d .* r)     (forward pre-smoothing residual; backward x2b = g - A (d .* g))
__device__ __forceinline__ void vc_smooth_res(int i0, int st, int n, const int32_t* __restrict__ rp,
                                              const int32_t* __restrict__ cols, const float* __restrict__ w,
                                              const float* __restrict__ d, const float* __restrict__ r,
                                              float* __restrict__ s) {
  for (int i = i0; i < n; i += st) {
    float acc = r[i];
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) {
      const int32_t j = cols[k];
      acc = fmaf(-w[k], d[j] * r[j], acc);
    }
    s[i] = acc;
  }
}

// y = (d ? d .* t : 0) + M x
__device__ __forceinline__ void vc_spmv(int i0, int st, int n, const int32_t* __restrict__ rp,
                                        const int32_t* __restrict__ cols, const float* __restrict__ w,
                                        const float* __restrict__ x, const float* __restrict__ d,
                                        const float* __restrict__ t, float* __restrict__ y) {
  for (int i = i0; i < n; i += st) {
    float acc = d ? d[i] * t[i] : 0.f;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) acc = fmaf(w[k], x[cols[k]], acc);
    y[i] = acc;
  }
}

// y = add + M x
__device__ __forceinline__ void vc_spmv_add(int i0, int st, int n, const int32_t* __restrict__ rp,
                                            const int32_t* __restrict__ cols, const float* __restrict__ w,
                                            const float* __restrict__ x, const float* __restrict__ add,
                                            float* __restrict__ y) {
  for (int i = i0; i < n; i += st) {
    float acc = add[i];
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) acc = fmaf(w[k], x[cols[k]], acc);
    y[i] = acc;
  }
}

// u = r - A x2 ; y = x2 + d .* u   (post-smoothing; u kept for the backward when non-null)
__device__ __forceinline__ void vc_post(int i0, int st, int n, const int32_t* __restrict__ rp,
                                        const int32_t* __restrict__ cols, const float* __restrict__ w,
                                        const float* __restrict__ d, const float* __restrict__ r,
                                        const float* __restrict__ x2, float* __restrict__ u, float* __restrict__ y) {
  for (int i = i0; i < n; i += st) {
    float acc = r[i];
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) acc = fmaf(-w[k], x2[cols[k]], acc);
    if (u) u[i] = acc;
    y[i] = fmaf(d[i], acc, x2[i]);
  }
}

// adjoint of the pre-smoothing: x1b = x2b - A sb ; rb = d .* (g + x1b) + sb
__device__ __forceinline__ void vc_pre_adjoint(int i0, int st, int n, const int32_t* __restrict__ rp,
                                               const int32_t* __restrict__ cols, const float* __restrict__ w,
                                               const float* __restrict__ d, const float* __restrict__ g,
                                               const float* __restrict__ x2b, const float* __restrict__ sb,
                                               float* __restrict__ x1b, float* __restrict__ rb) {
  for (int i = i0; i < n; i += st) {
    float acc = x2b[i];
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) acc = fmaf(-w[k], sb[cols[k]], acc);
    x1b[i] = acc;
    if (rb) rb[i] = fmaf(d[i], g[i] + acc, sb[i]);
  }
}

__global__ void k_vc_smooth_res(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                                const float* __restrict__ w, const float* __restrict__ d, const float* __restrict__ r,
                                float* __restrict__ s) {
  pdl_trigger();
  pdl_wait();
  const int64_t o = (int64_t)blockIdx.y * n;
  vc_smooth_res(blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, n, rp, cols, w, d, r + o, s + o);
}

__global__ void k_vc_post(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                          const float* __restrict__ w, const float* __restrict__ d, const float* __restrict__ r,
                          const float* __restrict__ x2, float* __restrict__ u, float* __restrict__ y) {
  pdl_trigger();
  pdl_wait();
  const int64_t o = (int64_t)blockIdx.y * n;
  vc_post(blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, n, rp, cols, w, d, r + o, x2 + o,
          u ? u + o : nullptr, y + o);
}

__global__ void k_vc_pre_adjoint(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                                 const float* __restrict__ w, const float* __restrict__ d, const float* __restrict__ g,
                                 const float* __restrict__ x2b, const float* __restrict__ sb, float* __restrict__ x1b,
                                 float* __restrict__ rb) {
  const int64_t o = (int64_t)blockIdx.y * n;
  vc_pre_adjoint(blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x, n, rp, cols, w, d, g + o, x2b + o,
                 sb + o, x1b + o, rb ? rb + o : nullptr);
}

}  // namespace afem

#include "afem_fact.cuh"

namespace afem {

// The coarse end of the V-cycle in ONE block per vector: levels lo..L-1 are
// small (<= kCoarseRows rows each), so their steps run back to back with
// block barriers instead of one launch each.
constexpr int kCoarseRows = 2048;
constexpr int kExactRows = 320;   // the first level below the finest of at most this many rows is solved exactly
constexpr int kCoarseBlock = 1024;

struct CoarseLevel {
  int n;
  const int32_t *a_rp, *a_cols, *pt_rp, *pt_cols, *p_rp, *p_cols;   // A_l, P_l^T (n_{l+1} rows), P_l (n_l rows)
  const float *a_w, *pt_w, *p_w, *d;
  // [B][n] buffers: t = the level's input r (l > lo), vs = s / sb, x2 = x2 / x2b,
  // u, w = the level's output x / rb (l > lo), g = the adjoint input, x1b
  float *t, *vs, *x2, *u, *w, *g, *x1b;
  // factored smoother (fact != 0): x1 = G r kept for the post-smoothing, wpre = L r,
  // wpost = L u, gpre = L x1b, gpost = L g, tmp = G g
  int fact;
  FactView f;
  float *x1, *wpre, *wpost, *gpre, *gpost, *tmp;
};
struct CoarsePlan {
  int lo, L;
  const float* minv;   // level L-1 solved exactly: x = minv r (row-major, symmetric), or nullptr
  CoarseLevel lev[kMaxLevels];
};

// y = M x for a dense row-major n x n M, one warp per row
__device__ __forceinline__ void dense_matvec(int n, const float* __restrict__ M, const float* __restrict__ x,
                                             float* __restrict__ y) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int i = w; i < n; i += nw) {
    const float* row = M + (int64_t)i * n;
    float acc = 0.f;
    for (int j = lane; j < n; j += 32) acc = fmaf(row[j], x[j], acc);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) y[i] = acc;
  }
}

// forward: x_lo = V_lo(r_lo), keeping t, u (and the factored smoothers' L r,
// L u) per level for the backward
__global__ void __launch_bounds__(kCoarseBlock) k_vc_coarse(CoarsePlan plan, const float* __restrict__ r_lo,
                                                            float* __restrict__ x_lo) {
  pdl_trigger();
  pdl_wait();
  const int64_t b = blockIdx.y;
  const int lo = plan.lo, L = plan.L, i0 = threadIdx.x, st = blockDim.x;
  for (int l = lo; l + 1 < L; ++l) {   // pre-smoothing residual, restriction
    const CoarseLevel& A = plan.lev[l];
    const CoarseLevel& C = plan.lev[l + 1];
    const int64_t o = b * A.n;
    const float* r = (l == lo ? r_lo : A.t) + o;
    float* s = A.vs + o;
    if (A.fact) {   // x1 = G r, s = r - A x1
      fact_lower(i0, st, A.f, r, A.wpre + o);
      __syncthreads();
      fact_upper(i0, st, A.f, A.wpre + o, nullptr, nullptr, A.x1 + o);
      __syncthreads();
      vc_res(i0, st, A.n, A.a_rp, A.a_cols, A.a_w, r, A.x1 + o, s);
    } else {
      vc_smooth_res(i0, st, A.n, A.a_rp, A.a_cols, A.a_w, A.d, r, s);
    }
    __syncthreads();
    vc_spmv(i0, st, C.n, A.pt_rp, A.pt_cols, A.pt_w, s, nullptr, nullptr, C.t + b * C.n);
    __syncthreads();
  }
  {
    const CoarseLevel& C = plan.lev[L - 1];
    const int64_t o = b * C.n;
    const float* r = (L - 1 == lo ? r_lo : C.t) + o;
    float* x = (L - 1 == lo ? x_lo : C.w) + o;
    if (plan.minv) {   // the exact level
      dense_matvec(C.n, plan.minv, r, x);
    } else if (C.fact) {
      fact_lower(i0, st, C.f, r, C.wpre + o);
      __syncthreads();
      fact_upper(i0, st, C.f, C.wpre + o, nullptr, nullptr, x);
    } else {
      for (int i = i0; i < C.n; i += st) x[i] = C.d[i] * r[i];
    }
    __syncthreads();
  }
  for (int l = L - 2; l >= lo; --l) {   // prolongation + x1, post-smoothing
    const CoarseLevel& A = plan.lev[l];
    const CoarseLevel& C = plan.lev[l + 1];
    const int64_t o = b * A.n;
    const float* r = (l == lo ? r_lo : A.t) + o;
    float* x2 = A.x2 + o;
    float* y = (l == lo ? x_lo : A.w) + o;
    if (A.fact) {   // x2 = x1 + P x_{l+1}; u = r - A x2; y = x2 + G u
      vc_spmv_add(i0, st, A.n, A.p_rp, A.p_cols, A.p_w, C.w + b * C.n, A.x1 + o, x2);
      __syncthreads();
      vc_res(i0, st, A.n, A.a_rp, A.a_cols, A.a_w, r, x2, A.u + o);
      __syncthreads();
      fact_lower(i0, st, A.f, A.u + o, A.wpost + o);
      __syncthreads();
      fact_upper(i0, st, A.f, A.wpost + o, nullptr, x2, y);
    } else {
      vc_spmv(i0, st, A.n, A.p_rp, A.p_cols, A.p_w, C.w + b * C.n, A.d, r, x2);
      __syncthreads();
      vc_post(i0, st, A.n, A.a_rp, A.a_cols, A.a_w, A.d, r, x2, A.u + o, y);
    }
    __syncthreads();
  }
}

// backward: from the adjoint g_lo of x_lo, rb_lo (the adjoint of r_lo), and
// per level g (the adjoint of the level's output) and x1b for the weights;
// on factored levels also L g (gpost) and L x1b (gpre)
__global__ void __launch_bounds__(kCoarseBlock) k_vc_coarse_adjoint(CoarsePlan plan, const float* __restrict__ g_lo,
                                                                    float* __restrict__ rb_lo) {
  const int64_t b = blockIdx.y;
  const int lo = plan.lo, L = plan.L, i0 = threadIdx.x, st = blockDim.x;
  for (int l = lo; l + 1 < L; ++l) {   // adjoint of the post-smoothing, then of the prolongation
    const CoarseLevel& A = plan.lev[l];
    const CoarseLevel& C = plan.lev[l + 1];
    const int64_t o = b * A.n;
    const float* g = (l == lo ? g_lo : A.g) + o;
    float* x2b = A.x2 + o;
    if (A.fact) {   // x2b = g - A G g
      fact_lower(i0, st, A.f, g, A.gpost + o);
      __syncthreads();
      fact_upper(i0, st, A.f, A.gpost + o, nullptr, nullptr, A.tmp + o);
      __syncthreads();
      vc_res(i0, st, A.n, A.a_rp, A.a_cols, A.a_w, g, A.tmp + o, x2b);
    } else {
      vc_smooth_res(i0, st, A.n, A.a_rp, A.a_cols, A.a_w, A.d, g, x2b);
    }
    __syncthreads();
    vc_spmv(i0, st, C.n, A.pt_rp, A.pt_cols, A.pt_w, x2b, nullptr, nullptr, C.g + b * C.n);
    __syncthreads();
  }
  {
    const CoarseLevel& C = plan.lev[L - 1];
    const int64_t o = b * C.n;
    const float* g = (L - 1 == lo ? g_lo : C.g) + o;
    float* rb = (L - 1 == lo ? rb_lo : C.w) + o;
    if (plan.minv) {   // the exact level: rb = minv g (symmetric), no parameter
      dense_matvec(C.n, plan.minv, g, rb);
    } else if (C.fact) {   // one use, out = G r: its adjoint terms as a pre-smoothing with x1b = g
      fact_lower(i0, st, C.f, g, C.gpre + o);
      __syncthreads();
      fact_upper(i0, st, C.f, C.gpre + o, nullptr, nullptr, rb);
    } else {
      for (int i = i0; i < C.n; i += st) rb[i] = C.d[i] * g[i];
    }
    __syncthreads();
  }
  for (int l = L - 2; l >= lo; --l) {   // adjoint of the restriction, then of the pre-smoothing
    const CoarseLevel& A = plan.lev[l];
    const CoarseLevel& C = plan.lev[l + 1];
    const int64_t o = b * A.n;
    const float* g = (l == lo ? g_lo : A.g) + o;
    float* sb = A.vs + o;
    float* rb = (l == lo ? rb_lo : A.w) + o;
    vc_spmv(i0, st, A.n, A.p_rp, A.p_cols, A.p_w, C.w + b * C.n, nullptr, nullptr, sb);
    __syncthreads();
    if (A.fact) {   // x1b = x2b - A sb ; rb = sb + G (g + x1b)
      vc_pre_adjoint(i0, st, A.n, A.a_rp, A.a_cols, A.a_w, A.d, g, A.x2 + o, sb, A.x1b + o, nullptr);
      __syncthreads();
      fact_lower(i0, st, A.f, A.x1b + o, A.gpre + o);
      __syncthreads();
      if (rb_lo || l != lo) fact_upper(i0, st, A.f, A.gpost + o, A.gpre + o, sb, rb);
    } else {
      vc_pre_adjoint(i0, st, A.n, A.a_rp, A.a_cols, A.a_w, A.d, g, A.x2 + o, sb, A.x1b + o,
                     (l == lo && !rb_lo) ? nullptr : rb);
    }
    __syncthreads();
  }
}

// Galerkin product C = P^T A P, one thread per coarse row I, on the caller's
// pattern of C: sum over the children i of I (row I of P^T), the entries
// A_ij of row i and the parents J of j (row j of P), in that fixed order, in
// FP64.  Also the FP32 copy and the l1 cap 2 / sum_J |C_IJ|.  An entry
// outside the pattern sets *missing.
__global__ void k_rap(int nc, const int32_t* __restrict__ pt_rp, const int32_t* __restrict__ pt_cols,
                      const float* __restrict__ pt_w, const int32_t* __restrict__ a_rp,
                      const int32_t* __restrict__ a_cols, const double* __restrict__ a_v,
                      const int32_t* __restrict__ p_rp, const int32_t* __restrict__ p_cols,
                      const float* __restrict__ p_w, const int32_t* __restrict__ c_rp,
                      const int32_t* __restrict__ c_cols, double* __restrict__ c_v, float* __restrict__ c_w,
                      float* __restrict__ cap, int* __restrict__ missing) {
  for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < nc; I += gridDim.x * blockDim.x) {
    const int32_t cb = c_rp[I], ce = c_rp[I + 1];
    for (int32_t k = cb; k < ce; ++k) c_v[k] = 0.0;
    for (int32_t kk = pt_rp[I]; kk < pt_rp[I + 1]; ++kk) {
      const int32_t i = pt_cols[kk];
      const double wi = pt_w[kk];
      for (int32_t ka = a_rp[i]; ka < a_rp[i + 1]; ++ka) {
        const int32_t j = a_cols[ka];
        const double aij = wi * a_v[ka];
        for (int32_t kp = p_rp[j]; kp < p_rp[j + 1]; ++kp) {
          const int32_t J = p_cols[kp];
          int32_t pos = cb;
          while (pos < ce && c_cols[pos] != J) ++pos;
          if (pos == ce) {
            atomicOr(missing, 1);
            continue;
          }
          c_v[pos] += aij * (double)p_w[kp];
        }
      }
    }
    double l1 = 0.0;
    for (int32_t k = cb; k < ce; ++k) {
      c_w[k] = (float)c_v[k];
      l1 += fabs(c_v[k]);
    }
    cap[I] = l1 > 0.0 ? (float)(2.0 / l1) : 0.f;
  }
}

// cap = 2 / sum_j |A_ij| for the level-0 matrix (0 on an empty row)
__global__ void k_l1cap(int n, const int32_t* __restrict__ rp, const double* __restrict__ vals,
                        float* __restrict__ cap) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double l1 = 0.0;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) l1 += fabs(vals[k]);
    cap[i] = l1 > 0.0 ? (float)(2.0 / l1) : 0.f;
  }
}

// per-sample energy sums: sums[b*4+0] += e . (A e), sums[b*4+1] += (e - z) . (A (e - z))
__global__ void k_energy_sums(int n, const float* __restrict__ z, const float* __restrict__ e,
                              const float* __restrict__ Ae, const float* __restrict__ Av, double* __restrict__ sums) {
  __shared__ double sh[32];
  const int64_t b = blockIdx.y;
  double ee = 0, vv = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int64_t k = b * n + i;
    const double ei = e[k];
    ee += ei * (double)Ae[k];
    vv += (ei - (double)z[k]) * (double)Av[k];
  }
  ee = block_sum(ee, sh);
  vv = block_sum(vv, sh);
  if (threadIdx.x == 0) {
    atomicAdd(&sums[b * 4], ee);
    atomicAdd(&sums[b * 4 + 1], vv);
  }
}

// v = e - z
__global__ void k_sub(int64_t n, const float* __restrict__ e, const float* __restrict__ z, float* __restrict__ v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = e[i] - z[i];
}

// dL/dz = -2 A (e - z) / (e . A e  B), in place over Av
__global__ void k_energy_grad(int n, int batch, const double* __restrict__ sums, float* __restrict__ Av) {
  const int64_t b = blockIdx.y;
  const double ee = sums[b * 4] > 0 ? sums[b * 4] : 1e-300;
  const float scale = (float)(-2.0 / (ee * batch));
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) Av[b * n + i] *= scale;
}

// dL/dc_l through d = cap sigmoid(c + logit 0.8):
//   dc_i = d_i (1 - d_i / cap_i) sum_b (g u + x1b r)   (coarsest level: sum_b g r)
__global__ void k_dc_vcycle(int n, int batch, const float* __restrict__ d, const float* __restrict__ cap,
                            const float* __restrict__ g, const float* __restrict__ u, const float* __restrict__ x1b,
                            const float* __restrict__ r, float* __restrict__ dc) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float acc = 0.f;
    for (int b = 0; b < batch; ++b) {
      const int64_t k = (int64_t)b * n + i;
      if (u) acc = fmaf(x1b[k], r[k], fmaf(g[k], u[k], acc));
      else acc = fmaf(g[k], r[k], acc);
    }
    const float di = d[i], ci = cap[i];
    dc[i] = ci > 0.f ? acc * di * (1.f - di / ci) : 0.f;
  }
}

// head backward: d o = dc (x) w (FP32 [n][64]); partials of dw = sum_i dc_i o_i and dbeta = sum_i dc_i
__global__ void k_head_backward(int n, const float* __restrict__ dc, const bf16* __restrict__ o,
                                const float* __restrict__ w, float* __restrict__ dO, float* __restrict__ part) {
  __shared__ float sh[kF + 1][8];
  float acc[kF + 1];
#pragma unroll
  for (int c = 0; c <= kF; ++c) acc[c] = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float g = dc[i];
    const __nv_bfloat162* row = reinterpret_cast<const __nv_bfloat162*>(o + (int64_t)i * kF);
    float2* drow = reinterpret_cast<float2*>(dO + (int64_t)i * kF);
#pragma unroll
    for (int c = 0; c < kF / 2; ++c) {
      const __nv_bfloat162 v = row[c];
      acc[2 * c] = fmaf(g, __low2float(v), acc[2 * c]);
      acc[2 * c + 1] = fmaf(g, __high2float(v), acc[2 * c + 1]);
      drow[c] = make_float2(g * w[2 * c], g * w[2 * c + 1]);
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

// G = dO (x) [O > 0] in BF16, and per-block column sums (db)
__global__ void k_relu_grad(int64_t M, const float* __restrict__ dO, const bf16* __restrict__ O,
                            bf16* __restrict__ G, float* __restrict__ db_part) {
  __shared__ float sh[kF][8];
  float acc0 = 0.f, acc1 = 0.f;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < M;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const __nv_bfloat162 o = reinterpret_cast<const __nv_bfloat162*>(O + row * kF)[lane];
    const float2 d = reinterpret_cast<const float2*>(dO + row * kF)[lane];
    const float g0 = __low2float(o) > 0.f ? d.x : 0.f, g1 = __high2float(o) > 0.f ? d.y : 0.f;
    reinterpret_cast<__nv_bfloat162*>(G + row * kF)[lane] = __floats2bfloat162_rn(g0, g1);
    acc0 += g0;
    acc1 += g1;
  }
  sh[2 * lane][w] = acc0;
  sh[2 * lane + 1][w] = acc1;
  __syncthreads();
  if (threadIdx.x < kF) {
    float s = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[threadIdx.x][k];
    db_part[(int64_t)blockIdx.x * kF + threadIdx.x] = s;
  }
}

// input layer backward: G_in = da (x) [a > 0]; partials of dW_in = x0^T G_in (2 x 64) and db_in
__global__ void k_input_backward(int64_t M, const float* __restrict__ da, const bf16* __restrict__ a,
                                 const float* __restrict__ x0, float* __restrict__ part) {
  __shared__ float sh[3 * kF][8];
  float acc[3][2] = {};
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; row < M;
       row += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const __nv_bfloat162 av = reinterpret_cast<const __nv_bfloat162*>(a + row * kF)[lane];
    const float2 d = reinterpret_cast<const float2*>(da + row * kF)[lane];
    const float g0 = __low2float(av) > 0.f ? d.x : 0.f, g1 = __high2float(av) > 0.f ? d.y : 0.f;
    const float f0 = x0[row * 2], f1 = x0[row * 2 + 1];
    acc[0][0] += f0 * g0; acc[0][1] += f0 * g1;
    acc[1][0] += f1 * g0; acc[1][1] += f1 * g1;
    acc[2][0] += g0;      acc[2][1] += g1;
  }
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    sh[q * kF + 2 * lane][w] = acc[q][0];
    sh[q * kF + 2 * lane + 1][w] = acc[q][1];
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 3 * kF; e += blockDim.x) {
    float s = 0.f;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += sh[e][k];
    part[(int64_t)blockIdx.x * 3 * kF + e] = s;
  }
}

// Adam on the FP32 master parameters.
__global__ void k_adam(int n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m1,
                       float* __restrict__ m2, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float a = b1 * m1[i] + (1 - b1) * gi;
    const float v = b2 * m2[i] + (1 - b2) * gi * gi;
    m1[i] = a;
    m2[i] = v;
    p[i] -= lr * (a / c1) / (sqrtf(v / c2) + eps);
  }
}

// W [k][n] FP32 -> Wt [n][k] and W [k][n] as BF16 (the two GEMM operand forms)
__global__ void k_weights_bf16(int nmat, const float* __restrict__ W, bf16* __restrict__ Wt, bf16* __restrict__ Wn) {
  const int total = nmat * kF * kF;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int m = e / (kF * kF), r = e % (kF * kF), k = r / kF, n = r % kF;
    const bf16 v = __float2bfloat16_rn(W[e]);
    Wt[m * kF * kF + n * kF + k] = v;
    Wn[e] = v;
  }
}

__global__ void k_f64_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

}  // namespace afem

// ---------------------------------------------------------------------------
// Network object.

using namespace afem;

namespace afem {
struct FcgWork;
static void free_fcg_work(FcgWork* w);   // defined with FcgWork (its destructor frees the captured graph)
}

struct CsrLevel {
  int nrow = 0, ncol = 0;
  int32_t* rp = nullptr;
  int32_t* cols = nullptr;
  float* w = nullptr;
  int64_t nnz = 0;
};

struct afem_mpnn_s {
  afem_context ctx = nullptr;
  int L = 0;                     // levels of the hierarchy (one head each)
  int NL = 0;                    // message-passing layers, on levels 0 .. NL-1
  int n[kMaxLevels] = {};
  CsrLevel S[kMaxLevels];        // aggregation graph per level (S[0] weights from A)
  CsrLevel R[kMaxLevels];        // restriction l -> l+1
  CsrLevel Rt[kMaxLevels];       // its transpose (backward)
  CsrLevel P[kMaxLevels];        // prolongation l+1 -> l
  CsrLevel Pt[kMaxLevels];       // its transpose (restriction of residuals)
  CsrLevel Ac[kMaxLevels];       // Galerkin operators A_l, FP32 values (Ac[0]: the matrix on the level-0 graph)
  double* ac64[kMaxLevels] = {};  // FP64 values of A_l, l >= 1
  int* missing = nullptr;        // set by k_rap when a product entry falls outside the caller's pattern
  int* tc_err = nullptr;         // set by k_row_gemm when one of its bounded mbarrier waits runs out
  int max_batch = 1;
  // parameters (FP32 master, flat): W_in[2][64], b_in[64], per layer W1, W2 [64][64], b[64],
  // then per level a head w[64], beta.  Levels l >= NL have no layer: o_l = h_l = R o_{l-1}.
  int nparam = 0;
  float* params = nullptr;
  float* grads = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  int adam_t = 0;
  bf16* Wt = nullptr;   // [2 NL][64][64] transposed BF16 (forward operands)
  bf16* Wn = nullptr;   // [2 NL][64][64] BF16 (backward dX operands)
  // operator
  double* diag = nullptr;
  double mean_log = 0;
  int n0 = 0;
  bool have_operator = false;
  bool scalings_valid = false;
  // network activations (batch 1: the features do not depend on r)
  float* x0 = nullptr;                       // [n0][2]
  bf16* a_in = nullptr;                      // [n0][64]
  bf16* h[kMaxLevels] = {};                  // layer inputs (h[0] = a_in)
  bf16* m[kMaxLevels] = {};                  // S h
  bf16* o[kMaxLevels] = {};                  // layer outputs
  float* dO[kMaxLevels] = {};                // FP32 d o per level [n][64]
  float* dH[kMaxLevels] = {};                // FP32 d h per level [n][64]
  bf16* Gb = nullptr;                        // BF16 G [n0][64]
  float* ftmp = nullptr;                     // FP32 [n0][64]
  // V-cycle
  float* base[kMaxLevels] = {};              // l1 cap 2 / ||row||_1 per level [n_l]
  float* d[kMaxLevels] = {};                 // learned smoother weights per level [n_l]
  float* dc[kMaxLevels] = {};                // dL/dc per level [n_l]
  float* t[kMaxLevels] = {};                 // level input r_l [B][n_l] (level 0: the caller's r, t0)
  const float* t0 = nullptr;
  int coarse_lo = 0;                         // levels coarse_lo..Lv-1 run in the coarse-levels kernels
  int ex = -1;                               // the level solved exactly (-1: none)
  int Lv = 0;                                // levels the V-cycle uses: ex + 1, or L
  float* minv = nullptr;                     // FP32 inverse of A_ex's nonzero rows' block [n_ex][n_ex]
  float* w[kMaxLevels] = {};                 // level output x_l (w[0] = M r in training); backward: rb_l
  float* s[kMaxLevels] = {};                 // adjoint g_l of the level output (s[0] = dL/dz)
  float* vs[kMaxLevels] = {};                // pre-smoothing residual s_l; backward: sb_l
  float* x2[kMaxLevels] = {};                // x1 + P x_{l+1}; backward: x2b_l
  float* u[kMaxLevels] = {};                 // post-smoothing residual (kept for the backward)
  float* x1b[kMaxLevels] = {};               // adjoint of the pre-smoothed x1
  double* sums = nullptr;                    // [B][4]
  float* part = nullptr;                     // partial sums (dW, db)
  int64_t part_cap = 0;
  float* a32 = nullptr;                      // A in FP32 on the level-0 graph (training loss)
  CsrLevel Aop;
  float* tmpB = nullptr;                     // [B][n0]
  float* r32 = nullptr;                      // FCG staging [n0]
  float* z32 = nullptr;                      // FCG staging [n0]
  // factored smoothers (the finest level and the levels of at most kFactRows rows)
  struct Fact {
    bool on = false;
    int k = -1;                                // edge head index
    int nlow = 0;
    int32_t *low_rp = nullptr, *lo_col = nullptr, *lo_row = nullptr, *up_rp = nullptr, *up_e = nullptr;
    int32_t* aidx = nullptr;                   // position of each lower edge in A_l's values
    float *a_low = nullptr, *lval = nullptr, *sq = nullptr, *z = nullptr, *m = nullptr, *dz = nullptr;
    float *gl_diag = nullptr, *gl_low = nullptr;
    float* scal = nullptr;                     // theta, bound, dL/dtheta
    int* istar = nullptr;
    unsigned long long* packed = nullptr;
    float *x1 = nullptr, *wpre = nullptr, *wpost = nullptr, *gpre = nullptr, *gpost = nullptr, *tmp = nullptr;
  } fl[kMaxLevels];
  int nfact = 0;
  afem::FcgWork* fcg = nullptr;              // FCG buffers and graph (created on first solve)
  bool pdl = false;                          // V-cycle kernels launched with programmatic dependent launch
  std::vector<void*> owned;
};

namespace afem {

static afem_status dalloc(afem_mpnn net, size_t bytes, void** out) {
  AFEM_CUDA(cudaMallocAsync(out, bytes, net->ctx->stream));
  net->owned.push_back(*out);
  return AFEM_OK;
}
template <class T>
static afem_status dalloc(afem_mpnn net, size_t count, T** out) {
  return dalloc(net, count * sizeof(T), reinterpret_cast<void**>(out));
}

static afem_status copy_csr(afem_mpnn net, CsrLevel& dst, int nrow, int ncol, const int32_t* rp, const int32_t* cols,
                            const float* w) {
  dst.nrow = nrow;
  dst.ncol = ncol;
  int32_t nnz = 0;
  AFEM_TRY(read_scalar(net->ctx, rp + nrow, &nnz));
  dst.nnz = nnz;
  AFEM_TRY(dalloc(net, (size_t)nrow + 1, &dst.rp));
  AFEM_TRY(dalloc(net, (size_t)std::max(nnz, 1), &dst.cols));
  AFEM_TRY(dalloc(net, (size_t)std::max(nnz, 1), &dst.w));
  cudaStream_t s = net->ctx->stream;
  AFEM_CUDA(cudaMemcpyAsync(dst.rp, rp, sizeof(int32_t) * (nrow + 1), cudaMemcpyDeviceToDevice, s));
  if (nnz) {
    AFEM_CUDA(cudaMemcpyAsync(dst.cols, cols, sizeof(int32_t) * nnz, cudaMemcpyDeviceToDevice, s));
    if (w) AFEM_CUDA(cudaMemcpyAsync(dst.w, w, sizeof(float) * nnz, cudaMemcpyDeviceToDevice, s));
  }
  return AFEM_OK;
}

// parameter offsets
static int off_win() { return 0; }
static int off_bin() { return 2 * kF; }
static int off_w1(int l) { return 3 * kF + l * (2 * kF * kF + kF); }
static int off_w2(int l) { return off_w1(l) + kF * kF; }
static int off_b(int l) { return off_w1(l) + 2 * kF * kF; }
static int off_head(int NL, int l) { return 3 * kF + NL * (2 * kF * kF + kF) + l * (kF + 1); }
static int off_edge(int NL, int L, int k) { return off_head(NL, L) + k * (kF + 1); }

// The factored smoother's index structures of level l from the pattern of
// A_l (host side, once): the strict lower entries in row order, their
// positions in A_l's values, and the transposed index by column.
static afem_status fact_setup(afem_mpnn net, int l, const CsrLevel& pat) {
  auto& f = net->fl[l];
  const int n = pat.nrow;
  cudaStream_t s = net->ctx->stream;
  std::vector<int32_t> rp(n + 1), cols(std::max<int64_t>(pat.nnz, 1));
  AFEM_CUDA(cudaMemcpyAsync(rp.data(), pat.rp, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost, s));
  if (pat.nnz) AFEM_CUDA(cudaMemcpyAsync(cols.data(), pat.cols, sizeof(int32_t) * pat.nnz, cudaMemcpyDeviceToHost, s));
  AFEM_CUDA(cudaStreamSynchronize(s));
  std::vector<int32_t> low_rp(n + 1, 0), lo_col, lo_row, aidx;
  for (int i = 0; i < n; ++i) {
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
      if (cols[k] < i) {
        lo_col.push_back(cols[k]);
        lo_row.push_back(i);
        aidx.push_back(k);
      }
    low_rp[i + 1] = (int32_t)lo_col.size();
  }
  const int nlow = (int)lo_col.size();
  std::vector<int32_t> up_rp(n + 1, 0), up_e(std::max(nlow, 1));
  for (int e = 0; e < nlow; ++e) ++up_rp[lo_col[e] + 1];
  for (int j = 0; j < n; ++j) up_rp[j + 1] += up_rp[j];
  {
    std::vector<int32_t> cur(up_rp.begin(), up_rp.end() - 1);
    for (int e = 0; e < nlow; ++e) up_e[cur[lo_col[e]]++] = e;   // rows ascending within a column
  }
  const size_t ne = std::max(nlow, 1), B = net->max_batch;
  f.on = true;
  f.nlow = nlow;
  AFEM_TRY(dalloc(net, (size_t)n + 1, &f.low_rp));
  AFEM_TRY(dalloc(net, (size_t)n + 1, &f.up_rp));
  AFEM_TRY(dalloc(net, ne, &f.lo_col));
  AFEM_TRY(dalloc(net, ne, &f.lo_row));
  AFEM_TRY(dalloc(net, ne, &f.up_e));
  AFEM_TRY(dalloc(net, ne, &f.aidx));
  for (float** p : {&f.a_low, &f.lval, &f.z, &f.m, &f.dz, &f.gl_low}) AFEM_TRY(dalloc(net, ne, p));
  for (float** p : {&f.sq, &f.gl_diag}) AFEM_TRY(dalloc(net, (size_t)n, p));
  for (float** p : {&f.x1, &f.wpre, &f.wpost, &f.gpre, &f.gpost, &f.tmp}) AFEM_TRY(dalloc(net, B * n, p));
  AFEM_TRY(dalloc(net, 4, &f.scal));
  AFEM_TRY(dalloc(net, 1, &f.istar));
  AFEM_TRY(dalloc(net, 1, &f.packed));
  AFEM_CUDA(cudaMemcpyAsync(f.low_rp, low_rp.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, s));
  AFEM_CUDA(cudaMemcpyAsync(f.up_rp, up_rp.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, s));
  if (nlow) {
    AFEM_CUDA(cudaMemcpyAsync(f.lo_col, lo_col.data(), sizeof(int32_t) * nlow, cudaMemcpyHostToDevice, s));
    AFEM_CUDA(cudaMemcpyAsync(f.lo_row, lo_row.data(), sizeof(int32_t) * nlow, cudaMemcpyHostToDevice, s));
    AFEM_CUDA(cudaMemcpyAsync(f.up_e, up_e.data(), sizeof(int32_t) * nlow, cudaMemcpyHostToDevice, s));
    AFEM_CUDA(cudaMemcpyAsync(f.aidx, aidx.data(), sizeof(int32_t) * nlow, cudaMemcpyHostToDevice, s));
  }
  AFEM_CUDA(cudaMemsetAsync(f.scal, 0, sizeof(float) * 4, s));
  AFEM_CUDA(cudaStreamSynchronize(s));   // the host vectors go out of scope
  return AFEM_OK;
}

static FactView fact_view(afem_mpnn net, int l) {
  const auto& f = net->fl[l];
  FactView v;
  v.n = net->n[l];
  v.nlow = f.nlow;
  v.low_rp = f.low_rp;
  v.lo_col = f.lo_col;
  v.lo_row = f.lo_row;
  v.up_rp = f.up_rp;
  v.up_e = f.up_e;
  v.lval = f.lval;
  v.sq = f.sq;
  v.theta = f.scal;
  return v;
}

static afem_status refresh_weights(afem_mpnn net) {
  afem_context ctx = net->ctx;
  const int L = net->NL;
  float* Wstack = nullptr;
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(float) * 2 * L * kF * kF)));
  AFEM_TRY(scratch_take(ctx, (size_t)2 * L * kF * kF, &Wstack));
  for (int l = 0; l < L; ++l) {
    AFEM_CUDA(cudaMemcpyAsync(Wstack + (2 * l) * kF * kF, net->params + off_w1(l), sizeof(float) * kF * kF,
                              cudaMemcpyDeviceToDevice, ctx->stream));
    AFEM_CUDA(cudaMemcpyAsync(Wstack + (2 * l + 1) * kF * kF, net->params + off_w2(l), sizeof(float) * kF * kF,
                              cudaMemcpyDeviceToDevice, ctx->stream));
  }
  net->scalings_valid = false;
  return launch(ctx, k_weights_bf16, grid_for(ctx, 2 * L * kF * kF, 256), 256, 0, 2 * L, (const float*)Wstack,
                net->Wt, net->Wn);
}

template <class TIn, class TOut>
static afem_status spmm(afem_mpnn net, const CsrLevel& S, const TIn* X, TOut* Y, int acc) {
  dim3 grid(grid_for(net->ctx, (int64_t)S.nrow * 32, 256, 8), 1);
  k_spmm<TIn, TOut><<<grid, 256, 0, net->ctx->stream>>>(S.nrow, S.ncol, S.rp, S.cols, S.w, X, (const bf16*)nullptr,
                                                        Y, acc);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_spmm", __FILE__, __LINE__);
  ++net->ctx->launches;
  return AFEM_OK;
}

// y = (dsc ? dsc .* tv : add, or 0) + M x, per vector of the batch
static afem_status sweep(afem_mpnn net, const CsrLevel* M, int batch, const float* x, const float* dsc,
                         const float* tv, float* y, int nrow, const float* add = nullptr) {
  dim3 grid(grid_for(net->ctx, nrow, 256, 8), batch);
  if (net->pdl)
    return M ? launch_pdl(net->ctx, net->ctx->stream, k_sweep, grid, 256, M->nrow, M->ncol, M->rp, M->cols, M->w, x,
                          dsc, tv, add, y)
             : launch_pdl(net->ctx, net->ctx->stream, k_sweep, grid, 256, nrow, 0, nullptr, nullptr, nullptr,
                          nullptr, dsc, tv, add, y);
  if (M)
    k_sweep<<<grid, 256, 0, net->ctx->stream>>>(M->nrow, M->ncol, M->rp, M->cols, M->w, x, dsc, tv, add, y);
  else
    k_sweep<<<grid, 256, 0, net->ctx->stream>>>(nrow, 0, nullptr, nullptr, nullptr, nullptr, dsc, tv, add, y);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_sweep", __FILE__, __LINE__);
  ++net->ctx->launches;
  return AFEM_OK;
}

// TMA descriptor of a row-major [rows x 64] BF16 matrix: 128-row boxes, 128-byte swizzle (the layout k_row_gemm's
// MMAs read); rows past the end read as zero.  cuTensorMapEncodeTiled comes from the CUDA driver through the
// runtime (cudaGetDriverEntryPointByVersion).
static afem_status rows64_map(const bf16* base, int64_t rows, CUtensorMap* map) {
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      fn = nullptr;
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode) return fail(AFEM_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the CUDA driver");
  const cuuint64_t dims[2] = {(cuuint64_t)kF, (cuuint64_t)std::max<int64_t>(rows, 1)};
  const cuuint64_t strides[1] = {(cuuint64_t)kF * sizeof(bf16)};
  const cuuint32_t box[2] = {(cuuint32_t)kF, (cuuint32_t)kTcRows};
  const cuuint32_t estride[2] = {1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<bf16*>(base), dims, strides, box,
                            estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(AFEM_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return AFEM_OK;
}

// Y = act(X1 B1 [+ X2 B2] + bias) over M rows on the tensor cores (k_row_gemm); at most 4 CTAs per SM
// (4 x 64 TMEM columns of the 512).
template <bool TWO, bool RELU>
static afem_status row_gemm_launch(afem_context ctx, int* err, int64_t M, const bf16* X1, const bf16* B1t,
                                   const bf16* X2, const bf16* B2t, const float* bias, bf16* Yb, float* Yf,
                                   int accumulate) {
  if (M <= 0) return AFEM_OK;
  CUtensorMap m1, m2;
  AFEM_TRY(rows64_map(X1, M, &m1));
  if (TWO) AFEM_TRY(rows64_map(X2, M, &m2));
  else m2 = m1;
  constexpr int smem = tc_smem_bytes<TWO>();
  static const cudaError_t attr = cudaFuncSetAttribute(k_row_gemm<TWO, RELU>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (attr != cudaSuccess) return cuda_fail(attr, "cudaFuncSetAttribute(k_row_gemm)", __FILE__, __LINE__);
  const int64_t tiles = (M + kTcRows - 1) / kTcRows;
  const unsigned grid = (unsigned)std::min<int64_t>(tiles, (int64_t)ctx->sm_count * (TWO ? 2 : 4));
  k_row_gemm<TWO, RELU><<<grid, 128, smem, ctx->stream>>>(m1, m2, (int)M, B1t, B2t, bias, Yb, Yf, accumulate, err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_row_gemm", __FILE__, __LINE__);
  ++ctx->launches;
  return AFEM_OK;
}

template <bool TWO, bool RELU>
static afem_status row_gemm(afem_mpnn net, int64_t M, const bf16* X1, const bf16* B1t, const bf16* X2,
                            const bf16* B2t, const float* bias, bf16* Yb, float* Yf, int accumulate) {
  return row_gemm_launch<TWO, RELU>(net->ctx, net->tc_err, M, X1, B1t, X2, B2t, bias, Yb, Yf, accumulate);
}

// Reports a timed-out tensor-core wait (k_row_gemm) as AFEM_ERR_TIMEOUT.  Reads the flag back (one small
// synchronous copy), except while the stream is being captured.
static afem_status check_tc(afem_mpnn net) {
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  AFEM_CUDA(cudaStreamIsCapturing(net->ctx->stream, &cs));
  if (cs != cudaStreamCaptureStatusNone) return AFEM_OK;
  int e = 0;
  AFEM_TRY(read_scalar(net->ctx, net->tc_err, &e));
  if (e) return fail(AFEM_ERR_TIMEOUT, "k_row_gemm: a tensor-core mbarrier wait ran out");
  return AFEM_OK;
}

// network forward on the coefficient features -> scalings d_l
// The factored smoother of level l from the level's weights d_l and output
// o_l: s = sqrt(d), the edge head and L's lower entries, then theta from the
// row sums of |L^T L A_l|.
static afem_status fact_values(afem_mpnn net, int l) {
  afem_context ctx = net->ctx;
  auto& f = net->fl[l];
  const int nl = net->n[l];
  const CsrLevel& A = net->Ac[l];
  AFEM_TRY(launch(ctx, k_fact_sq, grid_for(ctx, nl, 256, 8), 256, 0, nl, (const float*)net->d[l], f.sq));
  if (f.nlow)
    AFEM_TRY(launch(ctx, k_fact_edges, grid_for(ctx, f.nlow, 256, 8), 256, 0, f.nlow, (const int32_t*)f.lo_row,
                    (const int32_t*)f.lo_col, (const float*)f.a_low, (const bf16*)net->o[l],
                    (const float*)(net->params + off_edge(net->NL, net->L, f.k)), (const float*)f.sq, f.z, f.m,
                    f.lval));
  AFEM_CUDA(cudaMemsetAsync(f.packed, 0, sizeof(unsigned long long), ctx->stream));
  AFEM_TRY(launch(ctx, k_fact_rows, grid_for(ctx, nl, kFactRowBlock, 16), kFactRowBlock, 0, fact_view(net, l),
                  (const int32_t*)A.rp, (const int32_t*)A.cols, (const float*)A.w, f.packed));
  return launch(ctx, k_fact_theta, 1, 32, 0, (const unsigned long long*)f.packed, f.scal, f.scal + 1, f.istar);
}

static afem_status features_forward(afem_mpnn net) {
  afem_context ctx = net->ctx;
  const int n0 = net->n0, L = net->L;
  AFEM_TRY(launch(ctx, k_input_layer, grid_for(ctx, n0, 256, 8), 256, 0, n0, (const double*)net->diag, net->mean_log,
                  (const float*)(net->params + off_win()), (const float*)(net->params + off_bin()), net->x0,
                  net->a_in));
  for (int l = 0; l < L; ++l) {
    const int nl = net->n[l];
    if (l < net->NL) {
      AFEM_TRY(spmm<bf16, bf16>(net, net->S[l], net->h[l], net->m[l], 0));
      AFEM_TRY((row_gemm<true, true>(net, nl, net->h[l], net->Wt + (2 * l) * kF * kF, net->m[l],
                                     net->Wt + (2 * l + 1) * kF * kF, net->params + off_b(l), net->o[l], nullptr, 0)));
    }
    if (l + 1 < L) AFEM_TRY(spmm<bf16, bf16>(net, net->R[l], net->o[l], net->h[l + 1], 0));
    AFEM_TRY(launch(ctx, k_head, grid_for(ctx, nl, 256, 8), 256, 0, nl, (const bf16*)net->o[l],
                    (const float*)(net->params + off_head(net->NL, l)), (const float*)net->base[l], net->d[l]));
    if (net->fl[l].on) AFEM_TRY(fact_values(net, l));
  }
  AFEM_TRY(check_tc(net));
  net->scalings_valid = true;
  return AFEM_OK;
}

template <class Kernel, class... Args>
static afem_status launch_batch(afem_mpnn net, Kernel k, const char* name, int nrow, int batch, Args... args) {
  dim3 grid(grid_for(net->ctx, nrow, 256, 8), batch);
  if (net->pdl) return launch_pdl(net->ctx, net->ctx->stream, k, grid, 256, args...);
  k<<<grid, 256, 0, net->ctx->stream>>>(args...);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, name, __FILE__, __LINE__);
  ++net->ctx->launches;
  return AFEM_OK;
}

static CoarsePlan coarse_plan(afem_mpnn net) {
  CoarsePlan plan{};
  plan.lo = net->coarse_lo;
  plan.L = net->Lv;
  plan.minv = net->ex >= 0 ? net->minv : nullptr;
  for (int l = plan.lo; l < net->Lv; ++l) {
    CoarseLevel& c = plan.lev[l];
    c.n = net->n[l];
    c.a_rp = net->Ac[l].rp;
    c.a_cols = net->Ac[l].cols;
    c.a_w = net->Ac[l].w;
    c.d = net->d[l];
    c.t = net->t[l];
    c.vs = net->vs[l];
    c.x2 = net->x2[l];
    c.u = net->u[l];
    c.w = net->w[l];
    c.g = net->s[l];
    c.x1b = net->x1b[l];
    const auto& f = net->fl[l];
    c.fact = f.on;
    if (f.on) {
      c.f = fact_view(net, l);
      c.x1 = f.x1;
      c.wpre = f.wpre;
      c.wpost = f.wpost;
      c.gpre = f.gpre;
      c.gpost = f.gpost;
      c.tmp = f.tmp;
    }
    if (l + 1 < net->Lv) {
      c.pt_rp = net->Pt[l].rp;
      c.pt_cols = net->Pt[l].cols;
      c.pt_w = net->Pt[l].w;
      c.p_rp = net->P[l].rp;
      c.p_cols = net->P[l].cols;
      c.p_w = net->P[l].w;
    }
  }
  return plan;
}

// z = M r (one V-cycle) for `batch` FP32 vectors (r, z: [batch][n0]); with
// z == nullptr the result stays in w[0] and the states the backward needs
// (t, u per level) are kept
static afem_status apply(afem_mpnn net, int batch, const float* r, float* z) {
  const int lo = net->coarse_lo;
  const bool keep = z == nullptr;
  if (!net->scalings_valid) AFEM_TRY(features_forward(net));
  net->t0 = r;
  for (int l = 0; l < lo; ++l) {   // fine levels down: s = r - A (G r), r_{l+1} = P^T s
    const CsrLevel& A = net->Ac[l];
    const int nl = net->n[l];
    const float* rl = l == 0 ? r : net->t[l];
    const auto& f = net->fl[l];
    if (f.on) {   // x1 = G r = theta L^T (L r), s = r - A x1
      const FactView fv = fact_view(net, l);
      AFEM_TRY(launch_batch(net, k_fact_lower, "k_fact_lower", nl, batch, fv, rl, f.wpre));
      AFEM_TRY(launch_batch(net, k_fact_upper, "k_fact_upper", nl, batch, fv, (const float*)f.wpre,
                            (const float*)nullptr, (const float*)nullptr, f.x1));
      AFEM_TRY(launch_batch(net, k_vc_res, "k_vc_res", nl, batch, nl, (const int32_t*)A.rp, (const int32_t*)A.cols,
                            (const float*)A.w, rl, (const float*)f.x1, net->vs[l]));
    } else {
      AFEM_TRY(launch_batch(net, k_vc_smooth_res, "k_vc_smooth_res", nl, batch, nl, (const int32_t*)A.rp,
                            (const int32_t*)A.cols, (const float*)A.w, (const float*)net->d[l], rl, net->vs[l]));
    }
    AFEM_TRY(sweep(net, &net->Pt[l], batch, net->vs[l], nullptr, nullptr, net->t[l + 1], net->n[l + 1]));
  }
  float* x0 = z ? z : net->w[0];
  if (net->pdl) {
    AFEM_TRY(launch_pdl(net->ctx, net->ctx->stream, k_vc_coarse, dim3(1, batch), kCoarseBlock, coarse_plan(net),
                        lo == 0 ? r : (const float*)net->t[lo], lo == 0 ? x0 : net->w[lo]));
  } else {
    k_vc_coarse<<<dim3(1, batch), kCoarseBlock, 0, net->ctx->stream>>>(coarse_plan(net), lo == 0 ? r : net->t[lo],
                                                                      lo == 0 ? x0 : net->w[lo]);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "k_vc_coarse", __FILE__, __LINE__);
    ++net->ctx->launches;
  }
  for (int l = lo - 1; l >= 0; --l) {   // fine levels up: x2 = x1 + P x_{l+1}, post-smoothing
    const CsrLevel& A = net->Ac[l];
    const int nl = net->n[l];
    const float* rl = l == 0 ? r : net->t[l];
    float* y = l == 0 ? x0 : net->w[l];
    const auto& f = net->fl[l];
    if (f.on) {   // u = r - A x2, y = x2 + theta L^T (L u)
      const FactView fv = fact_view(net, l);
      AFEM_TRY(sweep(net, &net->P[l], batch, net->w[l + 1], nullptr, nullptr, net->x2[l], nl, f.x1));
      AFEM_TRY(launch_batch(net, k_vc_res, "k_vc_res", nl, batch, nl, (const int32_t*)A.rp, (const int32_t*)A.cols,
                            (const float*)A.w, rl, (const float*)net->x2[l], net->u[l]));
      AFEM_TRY(launch_batch(net, k_fact_lower, "k_fact_lower", nl, batch, fv, (const float*)net->u[l], f.wpost));
      AFEM_TRY(launch_batch(net, k_fact_upper, "k_fact_upper", nl, batch, fv, (const float*)f.wpost,
                            (const float*)nullptr, (const float*)net->x2[l], y));
    } else {
      AFEM_TRY(sweep(net, &net->P[l], batch, net->w[l + 1], net->d[l], rl, net->x2[l], nl));
      AFEM_TRY(launch_batch(net, k_vc_post, "k_vc_post", nl, batch, nl, (const int32_t*)A.rp,
                            (const int32_t*)A.cols, (const float*)A.w, (const float*)net->d[l], rl,
                            (const float*)net->x2[l], keep ? net->u[l] : (float*)nullptr, y));
    }
  }
  return AFEM_OK;
}

// dL/dc per level from the adjoint s[0] = dL/dz of the last training apply()
static afem_status apply_adjoint(afem_mpnn net, int batch) {
  afem_context ctx = net->ctx;
  const int lo = net->coarse_lo, L = net->L;
  for (int l = 0; l < lo; ++l) {   // adjoint of the post-smoothing, then of the prolongation
    const CsrLevel& A = net->Ac[l];
    const int nl = net->n[l];
    const auto& f = net->fl[l];
    if (f.on) {   // x2b = g - A G g, keeping L g
      const FactView fv = fact_view(net, l);
      AFEM_TRY(launch_batch(net, k_fact_lower, "k_fact_lower", nl, batch, fv, (const float*)net->s[l], f.gpost));
      AFEM_TRY(launch_batch(net, k_fact_upper, "k_fact_upper", nl, batch, fv, (const float*)f.gpost,
                            (const float*)nullptr, (const float*)nullptr, f.tmp));
      AFEM_TRY(launch_batch(net, k_vc_res, "k_vc_res", nl, batch, nl, (const int32_t*)A.rp, (const int32_t*)A.cols,
                            (const float*)A.w, (const float*)net->s[l], (const float*)f.tmp, net->x2[l]));
    } else {
      AFEM_TRY(launch_batch(net, k_vc_smooth_res, "k_vc_smooth_res", nl, batch, nl, (const int32_t*)A.rp,
                            (const int32_t*)A.cols, (const float*)A.w, (const float*)net->d[l],
                            (const float*)net->s[l], net->x2[l]));
    }
    AFEM_TRY(sweep(net, &net->Pt[l], batch, net->x2[l], nullptr, nullptr, net->s[l + 1], net->n[l + 1]));
  }
  {
    k_vc_coarse_adjoint<<<dim3(1, batch), kCoarseBlock, 0, ctx->stream>>>(coarse_plan(net), net->s[lo], net->w[lo]);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "k_vc_coarse_adjoint", __FILE__, __LINE__);
    ++ctx->launches;
  }
  for (int l = lo - 1; l >= 0; --l) {   // adjoint of the restriction, then of the pre-smoothing
    const CsrLevel& A = net->Ac[l];
    const int nl = net->n[l];
    const auto& f = net->fl[l];
    AFEM_TRY(sweep(net, &net->P[l], batch, net->w[l + 1], nullptr, nullptr, net->vs[l], nl));
    AFEM_TRY(launch_batch(net, k_vc_pre_adjoint, "k_vc_pre_adjoint", nl, batch, nl, (const int32_t*)A.rp,
                          (const int32_t*)A.cols, (const float*)A.w, (const float*)net->d[l], (const float*)net->s[l],
                          (const float*)net->x2[l], (const float*)net->vs[l], net->x1b[l],
                          (l == 0 || f.on) ? (float*)nullptr : net->w[l]));
    if (f.on) {   // L x1b, and rb = sb + theta L^T (L g + L x1b) above the finest level
      const FactView fv = fact_view(net, l);
      AFEM_TRY(launch_batch(net, k_fact_lower, "k_fact_lower", nl, batch, fv, (const float*)net->x1b[l], f.gpre));
      if (l > 0)
        AFEM_TRY(launch_batch(net, k_fact_upper, "k_fact_upper", nl, batch, fv, (const float*)f.gpost,
                              (const float*)f.gpre, (const float*)net->vs[l], net->w[l]));
    }
  }
  for (int l = 0; l < L; ++l) {
    if (net->fl[l].on) continue;   // fact_backward
    const int nl = net->n[l];
    if (l >= net->Lv || l == net->ex) {   // no smoother of the network on this level
      AFEM_CUDA(cudaMemsetAsync(net->dc[l], 0, sizeof(float) * nl, ctx->stream));
      continue;
    }
    const bool last = l == net->Lv - 1;
    AFEM_TRY(launch(ctx, k_dc_vcycle, grid_for(ctx, nl, 256, 8), 256, 0, nl, batch, (const float*)net->d[l],
                    (const float*)net->base[l], (const float*)net->s[l], last ? (const float*)nullptr : net->u[l],
                    last ? (const float*)nullptr : net->x1b[l], l == 0 ? net->t0 : (const float*)net->t[l],
                    net->dc[l]));
  }
  return AFEM_OK;
}

static afem_status ensure_part(afem_mpnn net, int64_t count) {
  if (count <= net->part_cap) return AFEM_OK;
  AFEM_TRY(dalloc(net, (size_t)count, &net->part));
  net->part_cap = count;
  return AFEM_OK;
}

static afem_status sum_partials(afem_context ctx, int nparts, int nelem, const float* part, float* dst,
                                int accumulate) {
  return launch(ctx, k_sum_partials, (unsigned)((nelem + 31) / 32), 32 * kSumWarps, 0, nparts, nelem, part, dst,
                accumulate);
}

// [dW1 ; dW2] = [X1^T G ; X2^T G] summed over M rows into dst (FP32 2 x 64 x 64, dW2 right after dW1),
// deterministic: per-CTA partials on the tensor cores (k_dw_grad), then a fixed-order sum
static int dw_grad_parts(afem_context ctx, int64_t M) {
  return (int)std::max<int64_t>(1, std::min<int64_t>((M + kTcRows - 1) / kTcRows, (int64_t)ctx->sm_count * 2));
}

// part: dw_grad_parts(ctx, M) x 2 x 64 x 64 floats
static afem_status dw_grad_launch(afem_context ctx, int* err, float* part, int64_t M, const bf16* X1,
                                  const bf16* X2, const bf16* G, float* dst) {
  if (M <= 0) return AFEM_OK;
  const int nb = dw_grad_parts(ctx, M);
  CUtensorMap m1, m2, mg;
  AFEM_TRY(rows64_map(X1, M, &m1));
  AFEM_TRY(rows64_map(X2, M, &m2));
  AFEM_TRY(rows64_map(G, M, &mg));
  static const cudaError_t attr = cudaFuncSetAttribute(k_dw_grad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                       kDwSmem);
  if (attr != cudaSuccess) return cuda_fail(attr, "cudaFuncSetAttribute(k_dw_grad)", __FILE__, __LINE__);
  k_dw_grad<<<nb, 128, kDwSmem, ctx->stream>>>(m1, m2, mg, (int)M, part, err);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "k_dw_grad", __FILE__, __LINE__);
  ++ctx->launches;
  return sum_partials(ctx, nb, 2 * kF * kF, (const float*)part, dst, 0);
}

static afem_status dw_gemm2(afem_mpnn net, int64_t M, const bf16* X1, const bf16* X2, const bf16* G, float* dst) {
  AFEM_TRY(ensure_part(net, (int64_t)dw_grad_parts(net->ctx, M) * 2 * kF * kF));
  return dw_grad_launch(net->ctx, net->tc_err, net->part, M, X1, X2, G, dst);
}

// loss and gradients of the mean relative squared error over (r, e)
// The factored levels' backward, after apply_adjoint: dL/dL (diagonal and
// lower entries) and dL/dtheta from the stored vectors, theta's term through
// its maximal row, then dL/dc of the level's weights, dz of the edge head and
// its parameter gradient.
static afem_status fact_backward(afem_mpnn net, int batch) {
  afem_context ctx = net->ctx;
  const int L = net->L;
  for (int l = 0; l < L; ++l) {
    auto& f = net->fl[l];
    if (!f.on) continue;
    const int nl = net->n[l];
    const bool last = l == net->Lv - 1;
    const FactView fv = fact_view(net, l);
    const float* rl = l == 0 ? net->t0 : net->t[l];
    const CsrLevel& A = net->Ac[l];
    const unsigned nbk = grid_for(ctx, nl, 256, 2);
    AFEM_TRY(ensure_part(net, std::max<int64_t>(nbk, (int64_t)grid_for(ctx, std::max(f.nlow, 1), 256, 2) * (kF + 1))));
    // the coarsest level's single use out = G r enters as a pre-smoothing with x1b = g
    AFEM_TRY(launch(ctx, k_fact_grad, nbk, 256, 0, fv, batch, rl, last ? (const float*)net->s[l] : net->x1b[l],
                    (const float*)f.wpre, (const float*)f.gpre, last ? (const float*)nullptr : net->u[l],
                    (const float*)net->s[l], (const float*)f.wpost, (const float*)f.gpost, f.gl_diag, f.gl_low,
                    net->part));
    AFEM_TRY(sum_partials(ctx, (int)nbk, 1, (const float*)net->part, f.scal + 2, 0));
    AFEM_TRY(launch(ctx, k_fact_theta_grad, 1, 32, 0, fv, (const int32_t*)A.rp, (const int32_t*)A.cols,
                    (const float*)A.w, (const float*)(f.scal + 1), (const int*)f.istar, (const float*)(f.scal + 2),
                    f.gl_diag, f.gl_low));
    AFEM_TRY(launch(ctx, k_fact_dc, grid_for(ctx, nl, 256, 8), 256, 0, fv, (const float*)f.m, (const float*)f.a_low,
                    (const float*)f.gl_diag, (const float*)f.gl_low, (const float*)net->d[l],
                    (const float*)net->base[l], net->dc[l]));
    float* gedge = net->grads + off_edge(net->NL, L, f.k);
    if (f.nlow) {
      const unsigned nbe = grid_for(ctx, f.nlow, 256, 2);
      AFEM_TRY(launch(ctx, k_fact_edge_backward, nbe, 256, 0, fv, (const float*)f.z, (const float*)f.a_low,
                      (const float*)f.gl_low, (const bf16*)net->o[l], f.dz, net->part));
      AFEM_TRY(sum_partials(ctx, (int)nbe, kF + 1, (const float*)net->part, gedge, 0));
    }
  }
  return AFEM_OK;
}

static afem_status loss_and_gradients(afem_mpnn net, int batch, const float* r, const float* e, double* loss_h) {
  afem_context ctx = net->ctx;
  cudaStream_t s = ctx->stream;
  const int n0 = net->n0, L = net->L;
  if (!net->scalings_valid) AFEM_TRY(features_forward(net));
  AFEM_TRY(apply(net, batch, r, nullptr));
  AFEM_CUDA(cudaMemsetAsync(net->sums, 0, sizeof(double) * 4 * batch, s));
  AFEM_CUDA(cudaMemsetAsync(net->grads, 0, sizeof(float) * net->nparam, s));
  // energy-norm loss ||(I - M A) e||_A^2 / ||e||_A^2: Av = A (e - z) into s[0], A e into tmpB
  AFEM_TRY(launch(ctx, k_sub, grid_for(ctx, (int64_t)batch * n0, 256), 256, 0, (int64_t)batch * n0, e,
                  (const float*)net->w[0], net->tmpB));
  AFEM_TRY(sweep(net, &net->Aop, batch, net->tmpB, nullptr, nullptr, net->s[0], n0));
  AFEM_TRY(sweep(net, &net->Aop, batch, e, nullptr, nullptr, net->tmpB, n0));
  {
    dim3 g(grid_for(ctx, n0, 256, 2), batch);
    k_energy_sums<<<g, 256, 0, s>>>(n0, net->w[0], e, net->tmpB, net->s[0], net->sums);
    k_energy_grad<<<g, 256, 0, s>>>(n0, batch, net->sums, net->s[0]);
    cudaError_t ce = cudaGetLastError();
    if (ce != cudaSuccess) return cuda_fail(ce, "k_energy", __FILE__, __LINE__);
    ctx->launches += 2;
  }
  // adjoint V-cycle -> dL/dc_l per level (and the factored levels' edge heads) ; heads
  AFEM_TRY(apply_adjoint(net, batch));
  AFEM_TRY(fact_backward(net, batch));
  for (int l = 0; l < L; ++l) {
    const int nl = net->n[l];
    const unsigned nbk = grid_for(ctx, nl, 256, 2);
    AFEM_TRY(ensure_part(net, (int64_t)nbk * (kF + 1)));
    AFEM_TRY(launch(ctx, k_head_backward, nbk, 256, 0, nl, (const float*)net->dc[l], (const bf16*)net->o[l],
                    (const float*)(net->params + off_head(net->NL, l)), net->dO[l], net->part));
    AFEM_TRY(sum_partials(ctx, (int)nbk, kF + 1, (const float*)net->part,
                    net->grads + off_head(net->NL, l), 0));
    const auto& f = net->fl[l];
    if (f.on && f.nlow)   // + the edge head's d o
      AFEM_TRY(launch(ctx, k_fact_dO, grid_for(ctx, (int64_t)nl * 32, 256, 8), 256, 0, fact_view(net, l),
                      (const float*)f.dz, (const bf16*)net->o[l],
                      (const float*)(net->params + off_edge(net->NL, L, f.k)), net->dO[l]));
  }
  // network backward, coarsest level first: o_l gets its head gradient plus R_l^T dh_{l+1}
  for (int l = L - 1; l >= 0; --l) {
    const int64_t M = net->n[l];
    if (l >= net->NL) {   // o_l = h_l = R_{l-1} o_{l-1}: pass the gradient down
      AFEM_TRY(spmm<float, float>(net, net->Rt[l - 1], net->dO[l], net->dO[l - 1], 1));
      continue;
    }
    const unsigned nbk = grid_for(ctx, M * 32, 256, 4);
    AFEM_TRY(ensure_part(net, std::max<int64_t>((int64_t)nbk * kF, (int64_t)ctx->sm_count * 2 * kF * kF)));
    AFEM_TRY(launch(ctx, k_relu_grad, nbk, 256, 0, M, (const float*)net->dO[l], (const bf16*)net->o[l], net->Gb,
                    net->part));
    AFEM_TRY(sum_partials(ctx, (int)nbk, kF, (const float*)net->part, net->grads + off_b(l), 0));
    AFEM_TRY(dw_gemm2(net, M, net->h[l], net->m[l], net->Gb, net->grads + off_w1(l)));   // dW2 at off_w2 = off_w1 + 64^2
    // dh_l = G W1^T + S_l^T (G W2^T)   (S_l symmetric)
    AFEM_TRY((row_gemm<false, false>(net, M, net->Gb, net->Wn + (2 * l) * kF * kF, nullptr, nullptr, nullptr,
                                     nullptr, net->dH[l], 0)));
    AFEM_TRY((row_gemm<false, false>(net, M, net->Gb, net->Wn + (2 * l + 1) * kF * kF, nullptr, nullptr, nullptr,
                                     nullptr, net->ftmp, 0)));
    AFEM_TRY(spmm<float, float>(net, net->S[l], net->ftmp, net->dH[l], 1));
    if (l > 0) AFEM_TRY(spmm<float, float>(net, net->Rt[l - 1], net->dH[l], net->dO[l - 1], 1));
  }
  {
    const unsigned nbk = grid_for(ctx, (int64_t)n0 * 32, 256, 4);
    AFEM_TRY(ensure_part(net, (int64_t)nbk * 3 * kF));
    AFEM_TRY(launch(ctx, k_input_backward, nbk, 256, 0, (int64_t)n0, (const float*)net->dH[0],
                    (const bf16*)net->a_in, (const float*)net->x0, net->part));
    AFEM_TRY(sum_partials(ctx, (int)nbk, 3 * kF, (const float*)net->part,
                    net->grads + off_win(), 0));
  }
  if (loss_h) {
    std::vector<double> hs(4 * batch);
    AFEM_CUDA(cudaMemcpyAsync(hs.data(), net->sums, sizeof(double) * 4 * batch, cudaMemcpyDeviceToHost, s));
    AFEM_CUDA(cudaStreamSynchronize(s));
    double l = 0;
    for (int b = 0; b < batch; ++b) l += hs[b * 4 + 1] / (hs[b * 4] + 1e-300);
    *loss_h = l / batch;
  }
  return check_tc(net);
}

}  // namespace afem

extern "C" {

afem_status afem_mpnn_create(afem_context ctx, int nb_levels, int nb_layers, const int* level_rows, const int32_t* const* graph_rp,
                             const int32_t* const* graph_cols, const float* const* graph_w,
                             const int32_t* const* restr_rp, const int32_t* const* restr_cols,
                             const float* const* restr_w, const int32_t* const* restrT_rp,
                             const int32_t* const* restrT_cols, const float* const* restrT_w,
                             const int32_t* const* prol_rp, const int32_t* const* prol_cols,
                             const float* const* prol_w, const int32_t* const* prolT_rp,
                             const int32_t* const* prolT_cols, const float* const* prolT_w,
                             const int32_t* const* coarse_rp, const int32_t* const* coarse_cols, int max_batch,
                             afem_mpnn* out) {
  AFEM_CHECK_ARG(ctx && out && level_rows, "afem_mpnn_create: null argument");
  AFEM_CHECK_ARG(nb_levels >= 1 && nb_levels <= kMaxLevels, "afem_mpnn_create: 1..%d levels", kMaxLevels);
  AFEM_CHECK_ARG(max_batch >= 1 && max_batch <= kMaxBatch, "afem_mpnn_create: max_batch 1..%d", kMaxBatch);
  AFEM_CHECK_ARG(nb_layers >= 1 && nb_layers <= nb_levels, "afem_mpnn_create: 1..%d layers", nb_levels);
  *out = nullptr;
  afem_mpnn net = new (std::nothrow) afem_mpnn_s();
  if (!net) return fail(AFEM_ERR_OOM, "afem_mpnn_create: host allocation");
  net->ctx = ctx;
  net->L = nb_levels;
  net->NL = nb_layers;
  net->max_batch = max_batch;
  auto cleanup = [&](afem_status st) {
    afem_mpnn_destroy(net);
    return st;
  };
  afem_status st;
  for (int l = 0; l < nb_levels; ++l) {
    net->n[l] = level_rows[l];
    if (level_rows[l] <= 0) return cleanup(fail(AFEM_ERR_BAD_ARG, "afem_mpnn_create: empty level %d", l));
    if ((st = copy_csr(net, net->S[l], level_rows[l], level_rows[l], graph_rp[l], graph_cols[l],
                       l == 0 ? nullptr : graph_w[l])) != AFEM_OK)
      return cleanup(st);
    if (l + 1 < nb_levels) {
      if ((st = copy_csr(net, net->R[l], level_rows[l + 1], level_rows[l], restr_rp[l], restr_cols[l], restr_w[l])) ||
          (st = copy_csr(net, net->Rt[l], level_rows[l], level_rows[l + 1], restrT_rp[l], restrT_cols[l],
                         restrT_w[l])) ||
          (st = copy_csr(net, net->P[l], level_rows[l], level_rows[l + 1], prol_rp[l], prol_cols[l], prol_w[l])) ||
          (st = copy_csr(net, net->Pt[l], level_rows[l + 1], level_rows[l], prolT_rp[l], prolT_cols[l], prolT_w[l])))
        return cleanup(st);
    }
    if (l > 0) {   // Galerkin pattern of A_l
      if (!coarse_rp || !coarse_cols || !coarse_rp[l] || !coarse_cols[l])
        return cleanup(fail(AFEM_ERR_BAD_ARG, "afem_mpnn_create: no coarse operator pattern for level %d", l));
      if ((st = copy_csr(net, net->Ac[l], level_rows[l], level_rows[l], coarse_rp[l], coarse_cols[l], nullptr)) ||
          (st = dalloc(net, (size_t)std::max<int64_t>(net->Ac[l].nnz, 1), &net->ac64[l])))
        return cleanup(st);
    }
  }
  net->n0 = level_rows[0];
  for (int l = 1; l < nb_levels && net->ex < 0; ++l)
    if (level_rows[l] <= kExactRows) net->ex = l;
  net->Lv = net->ex >= 0 ? net->ex + 1 : nb_levels;
  net->coarse_lo = net->Lv - 1;
  while (net->coarse_lo > 0 && level_rows[net->coarse_lo - 1] <= kCoarseRows) --net->coarse_lo;
  if (net->ex >= 0 && (st = dalloc(net, (size_t)level_rows[net->ex] * level_rows[net->ex], &net->minv)) != AFEM_OK)
    return cleanup(st);
  for (int l = 0; l < net->Lv; ++l) {
    if (l == net->ex || (l != 0 && level_rows[l] > kFactRows)) continue;
    if ((st = fact_setup(net, l, l == 0 ? net->S[0] : net->Ac[l])) != AFEM_OK) return cleanup(st);
    net->fl[l].k = net->nfact++;
  }
  net->nparam = off_edge(nb_layers, nb_levels, net->nfact);
  const size_t B = max_batch;
  const size_t n0 = net->n0;
  if ((st = dalloc(net, (size_t)net->nparam, &net->params)) || (st = dalloc(net, (size_t)net->nparam, &net->grads)) ||
      (st = dalloc(net, (size_t)net->nparam, &net->adam_m)) || (st = dalloc(net, (size_t)net->nparam, &net->adam_v)) ||
      (st = dalloc(net, (size_t)2 * nb_layers * kF * kF, &net->Wt)) ||
      (st = dalloc(net, (size_t)2 * nb_layers * kF * kF, &net->Wn)) || (st = dalloc(net, n0, &net->diag)) ||
      (st = dalloc(net, n0 * 2, &net->x0)) || (st = dalloc(net, n0 * kF, &net->a_in)) ||
      (st = dalloc(net, n0 * kF, &net->Gb)) || (st = dalloc(net, n0 * kF, &net->ftmp)) ||
      (st = dalloc(net, B * 4, &net->sums)) || (st = dalloc(net, n0, &net->r32)) || (st = dalloc(net, n0, &net->z32)) ||
      (st = dalloc(net, (size_t)std::max<int64_t>(net->S[0].nnz, 1), &net->a32)) || (st = dalloc(net, B * n0, &net->tmpB)) ||
      (st = dalloc(net, 1, &net->missing)) || (st = dalloc(net, 1, &net->tc_err)))
    return cleanup(st);
  if (cudaMemsetAsync(net->tc_err, 0, sizeof(int), net->ctx->stream) != cudaSuccess)
    return cleanup(fail(AFEM_ERR_CUDA, "afem_mpnn_create: cudaMemsetAsync"));
  net->h[0] = net->a_in;
  for (int l = 0; l < nb_levels; ++l) {
    const size_t nl = net->n[l];
    if (l > 0 && (st = dalloc(net, nl * kF, &net->h[l]))) return cleanup(st);
    if (l < nb_layers &&
        ((st = dalloc(net, nl * kF, &net->m[l])) || (st = dalloc(net, nl * kF, &net->o[l])) ||
         (st = dalloc(net, nl * kF, &net->dH[l]))))
      return cleanup(st);
    if (l >= nb_layers) net->o[l] = net->h[l];
    if ((st = dalloc(net, nl * kF, &net->dO[l])) ||
        (st = dalloc(net, nl, &net->base[l])) || (st = dalloc(net, nl, &net->d[l])) ||
        (st = dalloc(net, nl, &net->dc[l])) || (st = dalloc(net, B * nl, &net->t[l])) ||
        (st = dalloc(net, B * nl, &net->w[l])) || (st = dalloc(net, B * nl, &net->s[l])) ||
        (st = dalloc(net, B * nl, &net->vs[l])) || (st = dalloc(net, B * nl, &net->x2[l])) ||
        (st = dalloc(net, B * nl, &net->u[l])) || (st = dalloc(net, B * nl, &net->x1b[l])))
      return cleanup(st);
  }
  cudaStream_t s = ctx->stream;
  cudaMemsetAsync(net->adam_m, 0, sizeof(float) * net->nparam, s);
  cudaMemsetAsync(net->adam_v, 0, sizeof(float) * net->nparam, s);
  cudaMemsetAsync(net->params, 0, sizeof(float) * net->nparam, s);
  *out = net;
  return AFEM_OK;
}

afem_status afem_mpnn_destroy(afem_mpnn net) {
  if (!net) return AFEM_OK;
  cudaStream_t s = net->ctx->stream;
  free_fcg_work(net->fcg);
  for (void* p : net->owned) cudaFreeAsync(p, s);
  cudaStreamSynchronize(s);
  delete net;
  return AFEM_OK;
}

int afem_mpnn_param_count(afem_mpnn net) { return net ? net->nparam : 0; }

afem_status afem_mpnn_set_params(afem_mpnn net, const float* params_d) {
  AFEM_CHECK_ARG(net && params_d, "afem_mpnn_set_params: null argument");
  AFEM_CUDA(cudaMemcpyAsync(net->params, params_d, sizeof(float) * net->nparam, cudaMemcpyDeviceToDevice,
                            net->ctx->stream));
  net->adam_t = 0;
  AFEM_CUDA(cudaMemsetAsync(net->adam_m, 0, sizeof(float) * net->nparam, net->ctx->stream));
  AFEM_CUDA(cudaMemsetAsync(net->adam_v, 0, sizeof(float) * net->nparam, net->ctx->stream));
  return refresh_weights(net);
}

afem_status afem_mpnn_get_params(afem_mpnn net, float* params_d) {
  AFEM_CHECK_ARG(net && params_d, "afem_mpnn_get_params: null argument");
  AFEM_CUDA(cudaMemcpyAsync(params_d, net->params, sizeof(float) * net->nparam, cudaMemcpyDeviceToDevice,
                            net->ctx->stream));
  return AFEM_OK;
}

namespace afem {

// The exact level's inverse, on the host in FP64 once per operator: the block
// of A_ex's nonzero rows (the rows of coarse Dirichlet nodes are empty) by a
// Cholesky factorisation, inverted column by column, stored in FP32 with
// zeros on the empty rows and columns.
static afem_status exact_inverse(afem_mpnn net) {
  const int l = net->ex, n = net->n[l];
  const CsrLevel& A = net->Ac[l];
  cudaStream_t s = net->ctx->stream;
  std::vector<int32_t> rp(n + 1), cols(std::max<int64_t>(A.nnz, 1));
  std::vector<double> v(std::max<int64_t>(A.nnz, 1));
  AFEM_CUDA(cudaMemcpyAsync(rp.data(), A.rp, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToHost, s));
  if (A.nnz) {
    AFEM_CUDA(cudaMemcpyAsync(cols.data(), A.cols, sizeof(int32_t) * A.nnz, cudaMemcpyDeviceToHost, s));
    AFEM_CUDA(cudaMemcpyAsync(v.data(), net->ac64[l], sizeof(double) * A.nnz, cudaMemcpyDeviceToHost, s));
  }
  AFEM_CUDA(cudaStreamSynchronize(s));
  std::vector<int> act;   // the nonzero rows
  std::vector<int> pos(n, -1);
  for (int i = 0; i < n; ++i) {
    bool nz = false;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) nz |= v[k] != 0.0;
    if (nz) {
      pos[i] = (int)act.size();
      act.push_back(i);
    }
  }
  const int m = (int)act.size();
  std::vector<double> B((size_t)m * m, 0.0);
  for (int i = 0; i < n; ++i) {
    if (pos[i] < 0) continue;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k)
      if (pos[cols[k]] >= 0) B[(size_t)pos[i] * m + pos[cols[k]]] += v[k];
  }
  // B = C C^T (lower C in place)
  for (int j = 0; j < m; ++j) {
    double dj = B[(size_t)j * m + j];
    for (int k = 0; k < j; ++k) dj -= B[(size_t)j * m + k] * B[(size_t)j * m + k];
    if (!(dj > 0.0))
      return fail(AFEM_ERR_BREAKDOWN, "afem_mpnn_set_operator: the operator of level %d (solved exactly) is not "
                                      "positive definite", l);
    const double cj = std::sqrt(dj);
    B[(size_t)j * m + j] = cj;
    for (int i = j + 1; i < m; ++i) {
      double a = B[(size_t)i * m + j];
      for (int k = 0; k < j; ++k) a -= B[(size_t)i * m + k] * B[(size_t)j * m + k];
      B[(size_t)i * m + j] = a / cj;
    }
  }
  std::vector<float> out((size_t)n * n, 0.f);
  std::vector<double> y(m);
  for (int c = 0; c < m; ++c) {   // column c of B^-1: C y = e_c, C^T x = y
    for (int i = 0; i < m; ++i) {
      double a = i == c ? 1.0 : 0.0;
      for (int k = 0; k < i; ++k) a -= B[(size_t)i * m + k] * y[k];
      y[i] = a / B[(size_t)i * m + i];
    }
    for (int i = m - 1; i >= 0; --i) {
      double a = y[i];
      for (int k = i + 1; k < m; ++k) a -= B[(size_t)k * m + i] * y[k];
      y[i] = a / B[(size_t)i * m + i];
    }
    for (int i = 0; i < m; ++i) out[(size_t)act[i] * n + act[c]] = (float)y[i];
  }
  AFEM_CUDA(cudaMemcpyAsync(net->minv, out.data(), sizeof(float) * out.size(), cudaMemcpyHostToDevice, s));
  AFEM_CUDA(cudaStreamSynchronize(s));   // out goes out of scope
  return AFEM_OK;
}

}  // namespace afem

afem_status afem_mpnn_set_operator(afem_mpnn net, int n, const int32_t* rp, const int32_t* cols, const double* vals) {
  AFEM_CHECK_ARG(net && rp && cols && vals, "afem_mpnn_set_operator: null argument");
  AFEM_CHECK_ARG(n == net->n0, "afem_mpnn_set_operator: %d rows, network level 0 has %d", n, net->n0);
  int32_t nnz = 0;
  AFEM_TRY(read_scalar(net->ctx, rp + n, &nnz));
  AFEM_CHECK_ARG(nnz == net->S[0].nnz, "afem_mpnn_set_operator: matrix graph differs from level 0 (%d vs %lld nnz)",
                 nnz, (long long)net->S[0].nnz);
  afem_context ctx = net->ctx;
  cudaStream_t s = ctx->stream;
  AFEM_TRY(launch(ctx, k_diag, grid_for(ctx, n, 256), 256, 0, n, rp, cols, vals, net->diag));
  AFEM_TRY(launch(ctx, k_level0_weights, grid_for(ctx, n, 256), 256, 0, n, rp, cols, vals, (const double*)net->diag,
                  net->S[0].w));
  AFEM_TRY(launch(ctx, k_f64_to_f32, grid_for(ctx, nnz, 256), 256, 0, (int64_t)nnz, vals, net->a32));
  net->Aop = net->S[0];
  net->Aop.w = net->a32;
  // mean log diag (host, once per operator)
  {
    std::vector<double> hd(n);
    AFEM_CUDA(cudaMemcpyAsync(hd.data(), net->diag, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
    AFEM_CUDA(cudaStreamSynchronize(s));
    double acc = 0;
    for (int i = 0; i < n; ++i) acc += std::log(hd[i]);
    net->mean_log = acc / n;
  }
  // l1 caps and the Galerkin hierarchy A_{l+1} = P_l^T A_l P_l (FP64, FP32 copies)
  net->Ac[0] = net->Aop;
  AFEM_TRY(launch(ctx, k_l1cap, grid_for(ctx, n, 256), 256, 0, n, rp, vals, net->base[0]));
  AFEM_CUDA(cudaMemsetAsync(net->missing, 0, sizeof(int), s));
  for (int l = 1; l < net->L; ++l) {
    const CsrLevel& Pt = net->Pt[l - 1];
    const CsrLevel& P = net->P[l - 1];
    const CsrLevel& Af = net->Ac[l - 1];
    const double* af = l == 1 ? vals : net->ac64[l - 1];
    AFEM_TRY(launch(ctx, k_rap, grid_for(ctx, net->n[l], 128), 128, 0, net->n[l], (const int32_t*)Pt.rp,
                    (const int32_t*)Pt.cols, (const float*)Pt.w, (const int32_t*)Af.rp, (const int32_t*)Af.cols, af,
                    (const int32_t*)P.rp, (const int32_t*)P.cols, (const float*)P.w, (const int32_t*)net->Ac[l].rp,
                    (const int32_t*)net->Ac[l].cols, net->ac64[l], net->Ac[l].w, net->base[l], net->missing));
  }
  {
    int missing = 0;
    AFEM_CUDA(cudaMemcpyAsync(&missing, net->missing, sizeof(int), cudaMemcpyDeviceToHost, s));
    AFEM_CUDA(cudaStreamSynchronize(s));
    AFEM_CHECK_ARG(!missing, "afem_mpnn_set_operator: a coarse operator pattern misses entries of P^T A P");
  }
  if (net->ex >= 0) AFEM_TRY(exact_inverse(net));
  for (int l = 0; l < net->L; ++l) {   // the factored levels' lower entries of A_l (FP32)
    const auto& f = net->fl[l];
    if (!f.on || !f.nlow) continue;
    AFEM_TRY(launch(ctx, k_fact_gather, grid_for(ctx, f.nlow, 256), 256, 0, f.nlow, (const int32_t*)f.aidx,
                    (const float*)net->Ac[l].w, f.a_low));
  }
  net->have_operator = true;
  net->scalings_valid = false;
  return AFEM_OK;
}

afem_status afem_mpnn_forward(afem_mpnn net, int batch, const float* r_d, float* z_d) {
  AFEM_CHECK_ARG(net && r_d && z_d && batch >= 1 && batch <= net->max_batch, "afem_mpnn_forward: bad arguments");
  AFEM_CHECK_ARG(net->have_operator, "afem_mpnn_forward: call afem_mpnn_set_operator first");
  return apply(net, batch, r_d, z_d);
}

afem_status afem_mpnn_scalings(afem_mpnn net, int level, float* d_d) {
  AFEM_CHECK_ARG(net && d_d && level >= 0 && level < net->L, "afem_mpnn_scalings: bad arguments");
  AFEM_CHECK_ARG(net->have_operator, "afem_mpnn_scalings: call afem_mpnn_set_operator first");
  if (!net->scalings_valid) AFEM_TRY(features_forward(net));
  AFEM_CUDA(cudaMemcpyAsync(d_d, net->d[level], sizeof(float) * net->n[level], cudaMemcpyDeviceToDevice,
                            net->ctx->stream));
  return AFEM_OK;
}

afem_status afem_mpnn_gradients(afem_mpnn net, int batch, const float* r_d, const float* e_d, float* grad_d,
                                double* loss_h) {
  AFEM_CHECK_ARG(net && r_d && e_d && batch >= 1 && batch <= net->max_batch, "afem_mpnn_gradients: bad arguments");
  AFEM_CHECK_ARG(net->have_operator, "afem_mpnn_gradients: call afem_mpnn_set_operator first");
  AFEM_TRY(loss_and_gradients(net, batch, r_d, e_d, loss_h));
  if (grad_d)
    AFEM_CUDA(cudaMemcpyAsync(grad_d, net->grads, sizeof(float) * net->nparam, cudaMemcpyDeviceToDevice,
                              net->ctx->stream));
  return AFEM_OK;
}

afem_status afem_mpnn_train_step(afem_mpnn net, int batch, const float* r_d, const float* e_d, float lr,
                                 double* loss_h) {
  AFEM_TRY(afem_mpnn_gradients(net, batch, r_d, e_d, nullptr, loss_h));
  afem_context ctx = net->ctx;
  net->adam_t += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)net->adam_t), c2 = 1.f - powf(b2, (float)net->adam_t);
  AFEM_TRY(launch(ctx, k_adam, grid_for(ctx, net->nparam, 256), 256, 0, net->nparam, net->params,
                  (const float*)net->grads, net->adam_m, net->adam_v, lr, b1, b2, 1e-8f, c1, c2));
  return refresh_weights(net);
}

// The layer GEMMs on their own (testing, reuse).  Synchronous: they read back
// the kernels' error word.
afem_status afem_tc_row_gemm(afem_context ctx, int64_t M, const void* X1, const void* W1t, const void* X2,
                             const void* W2t, const float* bias, int relu, void* Yb, float* Yf, int accumulate) {
  AFEM_CHECK_ARG(ctx && M >= 0 && X1 && W1t && (Yb || Yf) && (!X2 == !W2t), "afem_tc_row_gemm: bad arguments");
  scratch_reset(ctx);
  AFEM_TRY(scratch_reserve(ctx, 256));
  int* err;
  AFEM_TRY(scratch_take(ctx, 1, &err));
  AFEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  const bf16 *x1 = static_cast<const bf16*>(X1), *w1 = static_cast<const bf16*>(W1t);
  const bf16 *x2 = static_cast<const bf16*>(X2), *w2 = static_cast<const bf16*>(W2t);
  bf16* yb = static_cast<bf16*>(Yb);
  if (X2 && relu) AFEM_TRY((row_gemm_launch<true, true>(ctx, err, M, x1, w1, x2, w2, bias, yb, Yf, accumulate)));
  else if (X2) AFEM_TRY((row_gemm_launch<true, false>(ctx, err, M, x1, w1, x2, w2, bias, yb, Yf, accumulate)));
  else if (relu) AFEM_TRY((row_gemm_launch<false, true>(ctx, err, M, x1, w1, x2, w2, bias, yb, Yf, accumulate)));
  else AFEM_TRY((row_gemm_launch<false, false>(ctx, err, M, x1, w1, x2, w2, bias, yb, Yf, accumulate)));
  int h = 0;
  AFEM_TRY(read_scalar(ctx, err, &h));
  if (h) return fail(AFEM_ERR_TIMEOUT, "afem_tc_row_gemm: a tensor-core mbarrier wait ran out");
  return AFEM_OK;
}

afem_status afem_tc_weight_grad(afem_context ctx, int64_t M, const void* X1, const void* X2, const void* G,
                                float* dW) {
  AFEM_CHECK_ARG(ctx && M >= 0 && X1 && X2 && G && dW, "afem_tc_weight_grad: bad arguments");
  const int nb = dw_grad_parts(ctx, M);
  scratch_reset(ctx);
  AFEM_TRY(scratch_reserve(ctx, 256 + align256(sizeof(float) * (size_t)nb * 2 * kF * kF)));
  int* err;
  float* part;
  AFEM_TRY(scratch_take(ctx, 1, &err));
  AFEM_TRY(scratch_take(ctx, (size_t)nb * 2 * kF * kF, &part));
  AFEM_CUDA(cudaMemsetAsync(err, 0, sizeof(int), ctx->stream));
  if (M == 0) AFEM_CUDA(cudaMemsetAsync(dW, 0, sizeof(float) * 2 * kF * kF, ctx->stream));
  AFEM_TRY(dw_grad_launch(ctx, err, part, M, static_cast<const bf16*>(X1), static_cast<const bf16*>(X2),
                          static_cast<const bf16*>(G), dW));
  int h = 0;
  AFEM_TRY(read_scalar(ctx, err, &h));
  if (h) return fail(AFEM_ERR_TIMEOUT, "afem_tc_weight_grad: a tensor-core mbarrier wait ran out");
  return AFEM_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Flexible CG (FCG(1): each new direction A-orthogonalised against the last
// one) with M as the preconditioner.  FP64 vectors, matrix, dot products and
// stop test; M runs in FP32 on r converted to FP32.  Scalars stay on the
// device (last-block reductions in a fixed order, deterministic); one
// iteration is 4 + (4 lo + 1) kernels (two per fine level each way, one
// coarse-levels kernel), captured in a CUDA graph per chunk of
// iterations, and a device flag makes the remaining kernels of a chunk return
// once converged.
//   K1  q = A p ; <p, q>, <r, p>            -> alpha = <r, p> / <p, q>
//   K2  x += alpha p ; r -= alpha q ; r32   -> <r, r>, stop test
//   M   z32 = M r32 (one V-cycle)
//   K3  z = z32 ; <z, q>                    -> beta = -<z, q> / <p, q>
//   K4  p = z + beta p

namespace afem {

struct FcgState {
  double pq, rp, alpha, beta, rr, bnorm2, tol2, pad;
  int done, iter, status, max_iter;
  unsigned int ticket[4];
};
static_assert(sizeof(FcgState) <= 256, "FcgState is read back through the context's 256-byte pinned buffer");

template <int G>
__global__ void __launch_bounds__(kSolveBlock) k_fcg_init(int n, const int32_t* __restrict__ rp,
                                                          const int32_t* __restrict__ cols,
                                                          const double* __restrict__ vals, const double* __restrict__ b,
                                                          const double* __restrict__ x, double* __restrict__ r,
                                                          float* __restrict__ r32, double* partials, FcgState* st,
                                                          double rtol, double atol, int max_iter,
                                                          const uint8_t* __restrict__ skip) {
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
    if (row < n && lane == 0) {
      const double bi = b[row], ri = bi - s;
      r[row] = ri;
      r32[row] = (float)ri;
      if (!(skip && skip[row])) {   // forced (penalty) rows stay out of both norms when skip is given
        rr += ri * ri;
        bb += bi * bi;
      }
    }
  }
  rr = block_sum(rr, sh);
  bb = block_sum(bb, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x * 2] = rr;
    partials[blockIdx.x * 2 + 1] = bb;
  }
  if (last_block(&st->ticket[0])) {
    const double trr = reduce_partials(partials, gridDim.x, 2, 0, sh);
    const double tbb = reduce_partials(partials, gridDim.x, 2, 1, sh);
    if (threadIdx.x == 0) {
      st->rr = trr;
      st->bnorm2 = tbb;
      st->tol2 = fmax(rtol * rtol * tbb, atol * atol);
      st->iter = 0;
      st->max_iter = max_iter;
      st->status = AFEM_OK;
      st->done = trr <= st->tol2 ? 1 : 0;
      st->ticket[0] = 0;
    }
  }
}

template <int G>
__global__ void __launch_bounds__(kSolveBlock) k_fcg_spmv(int n, const int32_t* __restrict__ rp,
                                                          const int32_t* __restrict__ cols,
                                                          const double* __restrict__ vals, const double* __restrict__ p,
                                                          const double* __restrict__ r, double* __restrict__ q,
                                                          double* partials, FcgState* st) {
  pdl_trigger();
  pdl_wait();
  if (((volatile FcgState*)st)->done) return;
  __shared__ double sh[kSolveBlock / 32];
  const int lane = threadIdx.x & (G - 1);
  const int groups = gridDim.x * (blockDim.x / G);
  const int nr = n + ((groups - n % groups) % groups);
  double pq = 0.0, rpd = 0.0;
  for (int row = (blockIdx.x * blockDim.x + threadIdx.x) / G; row < nr; row += groups) {
    double s = 0.0;
    if (row < n) s = row_dot<G>(row, rp, cols, vals, p, lane);
    else {
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
    }
    if (row < n && lane == 0) {
      const double pi = p[row];
      q[row] = s;
      pq += pi * s;
      rpd += r[row] * pi;
    }
  }
  pq = block_sum(pq, sh);
  rpd = block_sum(rpd, sh);
  if (threadIdx.x == 0) {
    partials[blockIdx.x * 2] = pq;
    partials[blockIdx.x * 2 + 1] = rpd;
  }
  if (last_block(&st->ticket[1])) {
    const double tpq = reduce_partials(partials, gridDim.x, 2, 0, sh);
    const double trp = reduce_partials(partials, gridDim.x, 2, 1, sh);
    if (threadIdx.x == 0) {
      st->pq = tpq;
      st->rp = trp;
      if (!(tpq > 0.0) || !isfinite(tpq)) {
        st->status = AFEM_ERR_BREAKDOWN;
        st->done = 1;
        st->alpha = 0.0;
      } else {
        st->alpha = trp / tpq;
      }
      st->ticket[1] = 0;
    }
  }
}

__global__ void __launch_bounds__(kSolveBlock) k_fcg_update(int n, double* __restrict__ x, double* __restrict__ r,
                                                            float* __restrict__ r32, const double* __restrict__ p,
                                                            const double* __restrict__ q, double* partials,
                                                            FcgState* st, const uint8_t* __restrict__ skip) {
  pdl_trigger();
  pdl_wait();
  if (((volatile FcgState*)st)->done) return;
  __shared__ double sh[kSolveBlock / 32];
  const double alpha = ((volatile FcgState*)st)->alpha;
  double rr = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    const double ri = r[i] - alpha * q[i];
    r[i] = ri;
    r32[i] = (float)ri;
    if (!(skip && skip[i])) rr += ri * ri;
  }
  rr = block_sum(rr, sh);
  if (threadIdx.x == 0) partials[blockIdx.x * 2] = rr;
  if (last_block(&st->ticket[2])) {
    const double trr = reduce_partials(partials, gridDim.x, 2, 0, sh);
    if (threadIdx.x == 0) {
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

// first != 0: p = z32 (the initial direction).  Otherwise z = z32 and
// <z, q> -> beta = -<z, q> / <p, q>.
__global__ void __launch_bounds__(kSolveBlock) k_fcg_widen(int n, const float* __restrict__ z32, double* __restrict__ z,
                                                           const double* __restrict__ q, double* __restrict__ p,
                                                           int first, double* partials, FcgState* st) {
  pdl_trigger();
  pdl_wait();
  if (((volatile FcgState*)st)->done) return;
  __shared__ double sh[kSolveBlock / 32];
  double zq = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double zi = (double)z32[i];
    if (first) {
      p[i] = zi;
    } else {
      z[i] = zi;
      zq += zi * q[i];
    }
  }
  if (first) return;
  zq = block_sum(zq, sh);
  if (threadIdx.x == 0) partials[blockIdx.x * 2] = zq;
  if (last_block(&st->ticket[3])) {
    const double t = reduce_partials(partials, gridDim.x, 2, 0, sh);
    if (threadIdx.x == 0) {
      st->beta = -t / st->pq;
      st->ticket[3] = 0;
    }
  }
}

__global__ void __launch_bounds__(kSolveBlock) k_fcg_dir(int n, const double* __restrict__ z, double* __restrict__ p,
                                                         const FcgState* st) {
  pdl_trigger();
  pdl_wait();
  if (((volatile const FcgState*)st)->done) return;
  const double beta = ((volatile const FcgState*)st)->beta;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = z[i] + beta * p[i];
}

// Solver buffers and the captured iteration graph, kept with the network and
// rebuilt when the operator or solution pointers change.
struct FcgWork {
  double *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *partials = nullptr;
  FcgState* st = nullptr;
  int nparts = 0;
  const void* key[5] = {};
  int key_chunk = 0;
  GraphChunk* graph = nullptr;    // `chunk` iterations
  GraphChunk* graph1 = nullptr;   // one iteration (the tail of a solve)
  int64_t launches_chunk = 0, launches_one = 0;   // kernels per replay of each
  ~FcgWork() {
    delete graph;
    delete graph1;
  }
};

static void free_fcg_work(FcgWork* w) { delete w; }

static afem_status fcg_work(afem_mpnn net, FcgWork** out) {
  if (!net->fcg) {
    FcgWork* w = new (std::nothrow) FcgWork();
    if (!w) return fail(AFEM_ERR_OOM, "afem_fcg_solve: host allocation");
    net->fcg = w;
    const size_t n = net->n0;
    w->nparts = (int)std::max<unsigned>(grid_for(net->ctx, (int64_t)n * 32, kSolveBlock, 8),
                                        grid_for(net->ctx, (int64_t)n, kSolveBlock, 8));
    AFEM_TRY(dalloc(net, n, &w->r));
    AFEM_TRY(dalloc(net, n, &w->z));
    AFEM_TRY(dalloc(net, n, &w->p));
    AFEM_TRY(dalloc(net, n, &w->q));
    AFEM_TRY(dalloc(net, (size_t)2 * w->nparts, &w->partials));
    AFEM_TRY(dalloc(net, sizeof(FcgState), reinterpret_cast<void**>(&w->st)));
    AFEM_CUDA(cudaMemsetAsync(w->st, 0, sizeof(FcgState), net->ctx->stream));
  }
  *out = net->fcg;
  return AFEM_OK;
}

// z32 = M r32 for one vector, launched on `stream` (the capture stream inside a graph)
static afem_status apply_on(afem_mpnn net, cudaStream_t stream) {
  afem_context ctx = net->ctx;
  cudaStream_t saved = ctx->stream;
  ctx->stream = stream;
  net->pdl = true;
  afem_status st = apply(net, 1, net->r32, net->z32);
  net->pdl = false;
  ctx->stream = saved;
  return st;
}

}  // namespace afem

extern "C" afem_status afem_fcg_solve(afem_context ctx, int n, const int32_t* rp, const int32_t* cols,
                                      const double* vals, const double* b, double* x, afem_mpnn net,
                                      const afem_solver_options* opt_in, afem_solve_info* info) {
  return afem::fcg_solve(ctx, n, rp, cols, vals, b, x, nullptr, net, opt_in, info);
}

// afem_fcg_solve with the forced-row mask `skip` (nullable) of a linear
// system: its rows stay out of the stop test's norms (skip_forced_rows).
afem_status afem::fcg_solve(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals,
                            const double* b, double* x, const uint8_t* skip, afem_mpnn net,
                            const afem_solver_options* opt_in, afem_solve_info* info) {
  AFEM_CHECK_ARG(ctx && n > 0 && rp && cols && vals && b && x && net, "afem_fcg_solve: bad arguments");
  AFEM_CHECK_ARG(net->ctx == ctx, "afem_fcg_solve: the network belongs to another context");
  AFEM_CHECK_ARG(net->n0 == n && net->have_operator, "afem_fcg_solve: network not set for this operator");
  afem_solver_options opt;
  if (opt_in) opt = *opt_in;
  else afem_solver_options_default(&opt);
  const int max_iter = opt.max_iter > 0 ? opt.max_iter : 1000;
  const int chunk = opt.check_every > 0 ? std::min(opt.check_every, 64) : 4;
  int32_t nnz32 = 0;
  AFEM_TRY(read_scalar(ctx, rp + n, &nnz32));
  const int G = lanes_per_row_fp64(n, nnz32);
  const unsigned grid_rows = grid_for(ctx, (int64_t)n * G, kSolveBlock, 8);
  const unsigned grid_vec = grid_for(ctx, n, kSolveBlock, 8);
  FcgWork* w = nullptr;
  AFEM_TRY(fcg_work(net, &w));
  if (!net->scalings_valid) AFEM_TRY(features_forward(net));
  const void* key[5] = {rp, cols, vals, x, skip};
  if (!w->graph || !w->graph1 || w->key_chunk != chunk || !std::equal(key, key + 5, w->key)) {
    delete w->graph;
    delete w->graph1;
    w->graph = new (std::nothrow) GraphChunk();
    w->graph1 = new (std::nothrow) GraphChunk();
    if (!w->graph || !w->graph1) return fail(AFEM_ERR_OOM, "afem_fcg_solve: host allocation");
    std::copy(key, key + 5, w->key);
    w->key_chunk = chunk;
    afem_status cst = AFEM_OK;
    const int64_t launches_start = ctx->launches;
    int64_t launches0 = launches_start;
    for (int gi = 0; gi < 2 && cst == AFEM_OK; ++gi) {
      const int iters = gi == 0 ? chunk : 1;
      cst = capture(ctx, gi == 0 ? *w->graph : *w->graph1, [&](cudaStream_t s) -> afem_status {
      for (int k = 0; k < iters; ++k) {
        AFEM_TRY(dispatch_g(G, [&](auto g) {
          return launch_pdl(ctx, s, k_fcg_spmv<decltype(g)::value>, dim3(grid_rows), kSolveBlock, n, rp, cols, vals,
                            (const double*)w->p, (const double*)w->r, w->q, w->partials, w->st);
        }));
        AFEM_TRY(launch_pdl(ctx, s, k_fcg_update, dim3(grid_vec), kSolveBlock, n, x, w->r, net->r32,
                            (const double*)w->p, (const double*)w->q, w->partials, w->st, skip));
        AFEM_TRY(apply_on(net, s));
        AFEM_TRY(launch_pdl(ctx, s, k_fcg_widen, dim3(grid_vec), kSolveBlock, n, (const float*)net->z32, w->z,
                            (const double*)w->q, w->p, 0, w->partials, w->st));
        AFEM_TRY(launch_pdl(ctx, s, k_fcg_dir, dim3(grid_vec), kSolveBlock, n, (const double*)w->z, w->p,
                            (const FcgState*)w->st));
      }
      return AFEM_OK;
    });
      (gi == 0 ? w->launches_chunk : w->launches_one) = ctx->launches - launches0;
      launches0 = ctx->launches;
    }
    ctx->launches = launches_start;   // counted when the graphs run
    if (cst != AFEM_OK) {
      delete w->graph;
      delete w->graph1;
      w->graph = w->graph1 = nullptr;
      return cst;
    }
  }
  cudaEvent_t e0, e1;
  AFEM_CUDA(cudaEventCreate(&e0));
  AFEM_CUDA(cudaEventCreate(&e1));
  AFEM_CUDA(cudaEventRecord(e0, ctx->stream));
  afem_status st = dispatch_g(G, [&](auto g) {
    return launch(ctx, k_fcg_init<decltype(g)::value>, grid_rows, kSolveBlock, 0, n, rp, cols, vals, b,
                  (const double*)x, w->r, net->r32, w->partials, w->st, opt.rtol, opt.atol, max_iter, skip);
  });
  if (st == AFEM_OK) st = apply(net, 1, net->r32, net->z32);
  if (st == AFEM_OK)
    st = launch(ctx, k_fcg_widen, grid_vec, kSolveBlock, 0, n, (const float*)net->z32, w->z, (const double*)w->q,
                w->p, 1, w->partials, w->st);
  // Chunks of `chunk` iterations while at least that many remain, then single
  // iterations: the remaining count is predicted from the residual's
  // reduction since the previous read-back (iterations past convergence
  // still launch their kernels, which only test the stop flag).
  FcgState hs{};
  double rr_prev = 0.0;
  int it_prev = 0;
  while (st == AFEM_OK) {
    cudaError_t ce = cudaMemcpyAsync(ctx->pinned, w->st, sizeof(FcgState), cudaMemcpyDeviceToHost, ctx->stream);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(ctx->stream);
    if (ce != cudaSuccess) {
      st = cuda_fail(ce, "afem_fcg_solve state", __FILE__, __LINE__);
      break;
    }
    hs = *reinterpret_cast<FcgState*>(ctx->pinned);
    if (hs.done) break;
    int left = chunk;   // launch a whole chunk unless fewer iterations are predicted
    if (hs.iter > it_prev && rr_prev > 0.0 && hs.rr > 0.0 && hs.rr < rr_prev && hs.tol2 > 0.0) {
      const double per_it = std::log(hs.rr / rr_prev) / (hs.iter - it_prev);   // log reduction of rr per iteration
      const double need = std::log(hs.tol2 / hs.rr) / per_it;
      if (need < chunk) left = std::max(1, (int)std::ceil(need - 1e-9));
    }
    rr_prev = hs.rr;
    it_prev = hs.iter;
    if (left >= chunk) {
      ce = cudaGraphLaunch(w->graph->exec, ctx->stream);
      ctx->launches += w->launches_chunk;
    } else {
      for (int k = 0; k < left && ce == cudaSuccess; ++k) {
        ce = cudaGraphLaunch(w->graph1->exec, ctx->stream);
        ctx->launches += w->launches_one;
      }
    }
    if (ce != cudaSuccess) {
      st = cuda_fail(ce, "cudaGraphLaunch", __FILE__, __LINE__);
      break;
    }
  }
  cudaEventRecord(e1, ctx->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st != AFEM_OK) return st;
  double rel = 0.0;
  AFEM_TRY(true_relres(ctx, n, rp, cols, vals, nnz32, b, x, skip, &rel));
  if (info) {
    info->iterations = hs.iter;
    info->refinements = 0;
    info->status = hs.status;
    info->relres = rel;
    info->solve_ms = ms;
  }
  if (hs.status == AFEM_ERR_NOT_CONVERGED)
    return fail(hs.status, "FCG did not reach the tolerance in %d iterations (relres %.3e)", hs.iter, rel);
  if (hs.status == AFEM_ERR_BREAKDOWN) return fail(hs.status, "FCG breakdown (<p, A p> <= 0 or non-finite)");
  return AFEM_OK;
}

// Levels of at most `rows` rows run in the coarse-levels kernel (one block
// per vector); the others one launch per V-cycle step.
extern "C" afem_status afem_mpnn_set_coarse_rows(afem_mpnn net, int rows) {
  AFEM_CHECK_ARG(net && rows >= 0, "afem_mpnn_set_coarse_rows: bad arguments");
  net->coarse_lo = net->Lv - 1;
  while (net->coarse_lo > 0 && net->n[net->coarse_lo - 1] <= rows) --net->coarse_lo;
  if (net->fcg) {   // the captured FCG iteration depends on the split
    delete net->fcg->graph;
    net->fcg->graph = nullptr;
  }
  return AFEM_OK;
}
