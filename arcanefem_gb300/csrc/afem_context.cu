// Context, errors, scratch arena and the device exclusive scan.
#include <cstdarg>
#include <cstring>

#include "afem_internal.cuh"

namespace afem {

static thread_local char g_last_error[512] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
}

afem_status fail(afem_status code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

afem_status cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
  set_error("CUDA error %s (%s) in %s at %s:%d", cudaGetErrorName(e), cudaGetErrorString(e), what, file, line);
  return e == cudaErrorMemoryAllocation ? AFEM_ERR_OOM : AFEM_ERR_CUDA;
}

afem_status check_flags(afem_context ctx) {
  int* h = reinterpret_cast<int*>(static_cast<char*>(ctx->pinned) + 256);
  AFEM_CUDA(cudaMemcpyAsync(h, ctx->flags_d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
  const int flags = *h;
  if (flags == 0) return AFEM_OK;
  AFEM_CUDA(cudaMemsetAsync(ctx->flags_d, 0, sizeof(int), ctx->stream));
  AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
  if (flags & kFlagDegenerateCell)
    return fail(AFEM_ERR_MESH, "degenerate cell: an element kernel met a cell of zero or non-finite measure "
                               "(volume, area or Jacobian determinant); its matrix entries are not finite");
  return fail(AFEM_ERR_CUDA, "unknown device flag 0x%x", flags);
}

afem_status scratch_reserve(afem_context ctx, size_t bytes) {
  ctx->scratch_used = 0;
  if (bytes <= ctx->scratch_cap) return AFEM_OK;
  size_t cap = bytes + bytes / 4 + (1 << 20);
  if (ctx->scratch) AFEM_CUDA(cudaFreeAsync(ctx->scratch, ctx->stream));
  ctx->scratch = nullptr;
  ctx->scratch_cap = 0;
  AFEM_CUDA(cudaMallocAsync((void**)&ctx->scratch, cap, ctx->stream));
  ctx->scratch_cap = cap;
  return AFEM_OK;
}

// ---------------------------------------------------------------------------
// Exclusive scan: tile of kScanTile = 256 threads x 8 items.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ int32_t block_exclusive_scan(int32_t v, int32_t* sh, int32_t* total) {
  // warp inclusive scan
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    int32_t s = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < (int)(blockDim.x >> 5)) sh[lane] = s;
  }
  __syncthreads();
  int32_t warp_prefix = w > 0 ? sh[w - 1] : 0;
  *total = sh[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_prefix + x - v;
}

// Phase 1: per-tile sums.
__global__ void k_scan_tile_sums(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ sums) {
  __shared__ int32_t sh[32];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += in[base + i];
  int32_t total;
  block_exclusive_scan(s, sh, &total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// Phase 3: scan inside each tile, offset by the scanned tile sum.
__global__ void k_scan_tiles(const int32_t* __restrict__ in, int64_t n, const int32_t* __restrict__ offsets,
                             int32_t* __restrict__ out, int write_total) {
  __shared__ int32_t sh[32];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int32_t v[kScanItems];
  int32_t s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0;
    s += v[i];
  }
  int32_t total;
  int32_t pre = block_exclusive_scan(s, sh, &total) + (offsets ? offsets[blockIdx.x] : 0);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = pre;
    pre += v[i];
  }
  if (write_total && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[n] = pre;
}

size_t scan_scratch_bytes(int64_t n) {
  size_t b = 0;
  while (n > kScanTile) {
    int64_t tiles = (n + kScanTile - 1) / kScanTile;
    b += 2 * align256(sizeof(int32_t) * (size_t)(tiles + 1));
    n = tiles;
  }
  return b + 256;
}

afem_status exclusive_scan_i32(afem_context ctx, const int32_t* in, int32_t* out, int64_t n) {
  if (n <= 0) {
    AFEM_CUDA(cudaMemsetAsync(out, 0, sizeof(int32_t), ctx->stream));
    return AFEM_OK;
  }
  int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) return launch(ctx, k_scan_tiles, 1, kScanThreads, 0, in, n, (const int32_t*)nullptr, out, 1);
  int32_t *sums, *offs;
  AFEM_TRY(scratch_take(ctx, (size_t)tiles + 1, &sums));
  AFEM_TRY(scratch_take(ctx, (size_t)tiles + 1, &offs));
  AFEM_TRY(launch(ctx, k_scan_tile_sums, (unsigned)tiles, kScanThreads, 0, in, n, sums));
  AFEM_TRY(exclusive_scan_i32(ctx, sums, offs, tiles));
  return launch(ctx, k_scan_tiles, (unsigned)tiles, kScanThreads, 0, in, n, (const int32_t*)offs, out, 1);
}

}  // namespace afem

using namespace afem;

extern "C" {

const char* afem_last_error(void) { return g_last_error; }

int afem_version(void) { return 10000; }

afem_status afem_context_create(afem_context* out, void* stream) {
  AFEM_CHECK_ARG(out != nullptr, "afem_context_create: null output");
  *out = nullptr;
  afem_context ctx = new (std::nothrow) afem_context_s();
  if (!ctx) return fail(AFEM_ERR_OOM, "afem_context_create: host allocation failed");
  ctx->stream = reinterpret_cast<cudaStream_t>(stream);
  cudaError_t e = cudaGetDevice(&ctx->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
  if (e == cudaSuccess) e = cudaMallocHost(&ctx->pinned, 512);
  if (e == cudaSuccess) e = cudaMalloc((void**)&ctx->flags_d, 256);
  if (e == cudaSuccess) e = cudaMemset(ctx->flags_d, 0, 256);
  if (e != cudaSuccess) {
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->flags_d) cudaFree(ctx->flags_d);
    delete ctx;
    return cuda_fail(e, "afem_context_create", __FILE__, __LINE__);
  }
  *out = ctx;
  return AFEM_OK;
}

afem_status afem_context_destroy(afem_context ctx) {
  if (!ctx) return AFEM_OK;
  cudaError_t e = cudaSuccess;
  if (ctx->scratch) e = cudaFreeAsync(ctx->scratch, ctx->stream);
  if (ctx->sp.buf) cudaFreeAsync(ctx->sp.buf, ctx->stream);
  cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
  if (ctx->copy_stream) {
    cudaStreamSynchronize(ctx->copy_stream);
    cudaStreamDestroy(ctx->copy_stream);
  }
  for (cudaEvent_t ev : ctx->chunk_ev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->h2d_stream) {
    cudaStreamSynchronize(ctx->h2d_stream);
    cudaStreamDestroy(ctx->h2d_stream);
  }
  for (cudaEvent_t ev : ctx->h2d_ev)
    if (ev) cudaEventDestroy(ev);
  if (ctx->pinned) cudaFreeHost(ctx->pinned);
  if (ctx->flags_d) cudaFree(ctx->flags_d);
  delete ctx;
  if (e != cudaSuccess) return cuda_fail(e, "afem_context_destroy", __FILE__, __LINE__);
  if (e2 != cudaSuccess) return cuda_fail(e2, "afem_context_destroy", __FILE__, __LINE__);
  return AFEM_OK;
}

afem_status afem_context_set_stream(afem_context ctx, void* stream) {
  AFEM_CHECK_ARG(ctx != nullptr, "afem_context_set_stream: null context");
  // make the old stream's scratch users finish before the new stream reuses it
  AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->stream = reinterpret_cast<cudaStream_t>(stream);
  return AFEM_OK;
}

afem_status afem_context_synchronize(afem_context ctx) {
  AFEM_CHECK_ARG(ctx != nullptr, "afem_context_synchronize: null context");
  AFEM_CUDA(cudaStreamSynchronize(ctx->stream));
  return check_flags(ctx);
}

afem_status afem_context_set_element_formulation(afem_context ctx, int formulation) {
  AFEM_CHECK_ARG(ctx != nullptr, "afem_context_set_element_formulation: null context");
  AFEM_CHECK_ARG(formulation == AFEM_FORMULATION_REFERENCE || formulation == AFEM_FORMULATION_TESTLAB ||
                     formulation == AFEM_FORMULATION_MINIMAL,
                 "afem_context_set_element_formulation: unknown formulation %d", formulation);
  ctx->formulation = formulation;
  return AFEM_OK;
}

afem_status afem_context_get_element_formulation(afem_context ctx, int* formulation_h) {
  AFEM_CHECK_ARG(ctx != nullptr && formulation_h != nullptr, "afem_context_get_element_formulation: null argument");
  *formulation_h = ctx->formulation;
  return AFEM_OK;
}

afem_status afem_context_launch_count(afem_context ctx, int64_t* count) {
  AFEM_CHECK_ARG(ctx != nullptr && count != nullptr, "afem_context_launch_count: null argument");
  *count = ctx->launches;
  return AFEM_OK;
}

}  // extern "C"
