// Internal helpers shared by the afem_gb300 translation units: the context
// (stream + scratch arena + launch counter), error reporting, and small
// device building blocks (warp/block reductions, exclusive scan).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/afem_gb300.h"

namespace afem {

constexpr int kSmCountDefault = 152;

// Bits of the context's device flag word (afem_context_s::flags_d), set by
// kernels and reported by the next synchronous call (check_flags).
constexpr int kFlagDegenerateCell = 1;   // an element kernel met a zero / non-finite cell measure

// ---------------------------------------------------------------------------
// Error reporting: the last message per host thread, status codes returned.
void set_error(const char* fmt, ...);
afem_status fail(afem_status code, const char* fmt, ...);
afem_status cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define AFEM_CUDA(call)                                                       \
  do {                                                                        \
    cudaError_t afem_e_ = (call);                                             \
    if (afem_e_ != cudaSuccess) return ::afem::cuda_fail(afem_e_, #call, __FILE__, __LINE__); \
  } while (0)

#define AFEM_CHECK_ARG(cond, ...)                                             \
  do {                                                                        \
    if (!(cond)) return ::afem::fail(AFEM_ERR_BAD_ARG, __VA_ARGS__);          \
  } while (0)

#define AFEM_TRY(...)                                                         \
  do {                                                                        \
    afem_status afem_s_ = (__VA_ARGS__);                                      \
    if (afem_s_ != AFEM_OK) return afem_s_;                                   \
  } while (0)

}  // namespace afem

// ---------------------------------------------------------------------------
// Context.
struct afem_context_s {
  cudaStream_t stream = nullptr;
  int device = 0;
  int sm_count = afem::kSmCountDefault;
  // scratch arena: one device buffer, bump-allocated inside one API call and
  // released as a whole at the start of the next (stream ordering keeps the
  // previous call's kernels ahead of any reuse).
  char* scratch = nullptr;
  size_t scratch_cap = 0;
  size_t scratch_used = 0;
  // pinned host staging for scalar read-backs
  void* pinned = nullptr;
  int64_t launches = 0;
  // device -> host copies overlapped with kernels (afem_gather_to_host),
  // created on first use
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t chunk_ev[17] = {};
  // host -> device coordinate uploads overlapped with kernels (afem_assemble_host_io), created on first use
  cudaStream_t h2d_stream = nullptr;
  cudaEvent_t h2d_ev[17] = {};
  // The rows, ascending and at padded offsets, and the slot map that
  // afem_sparsity_rows found, kept for the next afem_sparsity_cols on the same
  // mesh arrays (which then only copies them into place).
  struct SparsityRows {
    void* buf = nullptr;
    size_t cap = 0;
    int32_t* cols = nullptr;   // row n at (npc - 1) * nc_ptr[n] + n
    int32_t* len = nullptr;    // [nb_node + 1] row lengths
    uint8_t* slot = nullptr;   // [incidences * npc]
    const int32_t* cn = nullptr;
    const int32_t* nc_ptr = nullptr;
    const int32_t* nc_cell = nullptr;
    int nb_node = 0, npc = 0;
    int64_t incidences = 0;
    bool valid = false;
  } sp;
  // element arithmetic of the assembly kernels (AFEM_FORMULATION_*)
  int formulation = AFEM_FORMULATION_REFERENCE;
  // device flag word (afem::kFlag*), set by kernels, read and cleared by check_flags
  int* flags_d = nullptr;
};

namespace afem {

// Reset the arena (call at the start of each public entry point that uses it).
inline void scratch_reset(afem_context ctx) { ctx->scratch_used = 0; }

// Reserve `bytes` for the whole call before any bump allocation, so that the
// arena is not reallocated while earlier pointers of the same call are live.
afem_status scratch_reserve(afem_context ctx, size_t bytes);

// Bump-allocate from the reserved arena (256-byte aligned).
template <class T>
afem_status scratch_take(afem_context ctx, size_t count, T** out) {
  size_t bytes = (count * sizeof(T) + 255) & ~size_t(255);
  if (ctx->scratch_used + bytes > ctx->scratch_cap)
    return fail(AFEM_ERR_OOM, "scratch arena overflow (%zu + %zu > %zu)", ctx->scratch_used, bytes,
                ctx->scratch_cap);
  *out = reinterpret_cast<T*>(ctx->scratch + ctx->scratch_used);
  ctx->scratch_used += bytes;
  return AFEM_OK;
}

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Launch helper: grid-stride launches, error check, launch accounting.
template <class Kernel, class... Args>
afem_status launch(afem_context ctx, Kernel k, unsigned grid, unsigned block, size_t smem, Args... args) {
  if (grid == 0) return AFEM_OK;
  k<<<grid, block, smem, ctx->stream>>>(args...);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch", __FILE__, __LINE__);
  ++ctx->launches;
  return AFEM_OK;
}

inline unsigned grid_for(afem_context ctx, int64_t work_items, int block, int max_blocks_per_sm = 8) {
  int64_t need = (work_items + block - 1) / block;
  int64_t cap = (int64_t)ctx->sm_count * max_blocks_per_sm;
  if (need > cap) need = cap;
  if (need < 1) need = 1;
  return (unsigned)need;
}

// Report (and clear) the flags kernels set since the last check: waits for the
// context stream.  AFEM_ERR_MESH for a degenerate cell.
afem_status check_flags(afem_context ctx);

// Read one device value into host memory (synchronous on the stream).
template <class T>
afem_status read_scalar(afem_context ctx, const T* d, T* h) {
  AFEM_CUDA(cudaMemcpyAsync(ctx->pinned, d, sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
  AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
  *h = *reinterpret_cast<T*>(ctx->pinned);
  return AFEM_OK;
}

// y = A x (FP64 CSR), lanes per row chosen from nnz / n (afem_solver.cu).
afem_status spmv_fp64(afem_context ctx, int n, int64_t nnz, const int32_t* rp, const int32_t* cols,
                      const double* vals, const double* x, double* y);

// afem_fcg_solve with a forced-row mask (nullable) for the stop test's norms
// (afem_mpnn.cu); the linear system's learned-preconditioner solve.
afem_status fcg_solve(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals,
                      const double* b, double* x, const uint8_t* skip, afem_mpnn net,
                      const afem_solver_options* opt, afem_solve_info* info);

// Exclusive scan of int32 counts into int32 offsets out[0..n] (out[n] = total),
// three-phase (tile sums, scan of sums, add-back), deterministic.
// Needs scan_scratch_bytes(n) bytes of scratch.
size_t scan_scratch_bytes(int64_t n);
afem_status exclusive_scan_i32(afem_context ctx, const int32_t* in, int32_t* out, int64_t n);

// ---------------------------------------------------------------------------
// Device helpers.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum (result valid in thread 0). `sh` needs blockDim/32 doubles.
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  int nw = blockDim.x >> 5;
  v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0) v = warp_sum(v);
  __syncthreads();
  return v;
}

// Block-wide sum of FP32 per-thread partials: warp sums in FP32, warp totals
// summed in FP64 (result valid in thread 0).  Keeps per-element dot-product
// work off GB300's narrow FP64 pipe.
__device__ __forceinline__ double block_sum_f(float v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = (double)v;
  __syncthreads();
  int nw = blockDim.x >> 5;
  double d = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
  if (w == 0) d = warp_sum(d);
  __syncthreads();
  return d;
}

}  // namespace afem
