// Shared pieces of the Krylov solvers (CG, mixed-precision CG, flexible CG
// with the learned preconditioner): G-lanes-per-row CSR dot products,
// deterministic last-block reductions, the lanes-per-row choice, sliced-ELL
// matrix copies, and CUDA graph capture of a chunk of iterations.
#pragma once
#include <type_traits>

#include "afem_internal.cuh"

namespace afem {

constexpr int kSolveBlock = 256;

// ---------------------------------------------------------------------------
// SpMV: G lanes per row, fixed-order reduction.
// Thread-per-row form: the row is read in chunks of kRowChunk entries whose
// column and value loads are all issued before their gathers (predicated past
// the row end with a zero weight on the row's own entry), so a thread keeps
// kRowChunk loads in flight.  Entries are summed in increasing k order.
// A negative column marks an unused slot of a reference CSR view
// (femutils/CsrFormatMatrix.cc:49-50): it gets the same zero weight, so the
// row's sum is that of its used entries.
constexpr int kRowChunk = 8;

template <class Acc, class T, class V>
__device__ __forceinline__ Acc row_dot_chunked(int row, const int32_t* __restrict__ rp,
                                               const int32_t* __restrict__ cols, const T* __restrict__ vals,
                                               const V* __restrict__ x) {
  Acc s = Acc(0);
  const int32_t e = __ldg(rp + row + 1);
  for (int32_t k = __ldg(rp + row); k < e; k += kRowChunk) {
    int32_t c[kRowChunk];
    T a[kRowChunk];
#pragma unroll
    for (int u = 0; u < kRowChunk; ++u) {
      const int32_t cc = k + u < e ? __ldg(cols + k + u) : -1;
      const bool in = cc >= 0;
      c[u] = in ? cc : row;
      a[u] = in ? __ldg(vals + k + u) : T(0);
    }
#pragma unroll
    for (int u = 0; u < kRowChunk; ++u) s += (Acc)a[u] * (Acc)__ldg(x + c[u]);
  }
  return s;
}

template <int G, class T, class V>
__device__ __forceinline__ double row_dot(int row, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                                          const T* __restrict__ vals, const V* __restrict__ x, int lane) {
  if constexpr (G == 1) return row_dot_chunked<double>(row, rp, cols, vals, x);
  double s = 0.0;
  const int32_t e = __ldg(rp + row + 1);
  for (int32_t k = __ldg(rp + row) + lane; k < e; k += G) {
    const int32_t c = __ldg(cols + k);
    if (c >= 0) s += (double)__ldg(vals + k) * (double)__ldg(x + c);
  }
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o, G);
  return s;
}

// ---------------------------------------------------------------------------
// Last-block finalize helper: every block publishes partials[blockIdx.x * W + w];
// returns true in the (single) last block, after which all partials are visible.
__device__ __forceinline__ bool last_block(unsigned int* ticket) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned int t = atomicAdd(ticket, 1u);
    is_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (is_last) __threadfence();
  return is_last;
}

// Fixed-order sum of partials[k * W + w], k < nparts (valid in thread 0).
__device__ __forceinline__ double reduce_partials(const double* partials, int nparts, int W, int w, double* sh) {
  double s = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) s += ((volatile const double*)partials)[(int64_t)k * W + w];
  return block_sum(s, sh);
}

// ---------------------------------------------------------------------------
// Host side.

// FP64 rows: on GB300 a warp FP64 instruction costs the same whatever its
// active lanes, so the shuffle-tree reduction and the lane-0 dot-product
// updates of a lanes-per-row layout multiply the FP64 issue count (measured:
// the FP64 pipe, not HBM, bound an 8-lane FP64 SpMV).  Short FP64 rows are
// therefore processed one thread per row, longer ones with few lanes.
inline int lanes_per_row_fp64(int n, int64_t nnz) {
  const double avg = n > 0 ? (double)nnz / n : 1.0;
  if (avg <= 24) return 1;
  if (avg <= 96) return 4;
  return 8;
}

template <class F>
afem_status dispatch_g(int G, F&& f) {
  switch (G) {
    case 1: return f(std::integral_constant<int, 1>{});
    case 2: return f(std::integral_constant<int, 2>{});
    case 4: return f(std::integral_constant<int, 4>{});
    case 8: return f(std::integral_constant<int, 8>{});
    case 16: return f(std::integral_constant<int, 16>{});
    default: return f(std::integral_constant<int, 32>{});
  }
}

template <class Kernel, class... Args>
inline afem_status launch_s(afem_context ctx, cudaStream_t s, Kernel k, unsigned grid, unsigned block, Args... args) {
  k<<<grid, block, 0, s>>>(args...);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch", __FILE__, __LINE__);
  ++ctx->launches;
  return AFEM_OK;
}

// Programmatic dependent launch.  A kernel launched with launch_pdl may
// start while its predecessor in the stream is still running; it must call
// pdl_wait() before touching anything the predecessor writes (the wait
// returns once that grid has completed and its memory is visible).
// pdl_trigger() lets the next such kernel begin launching early.  Both are
// no-ops for a kernel launched the ordinary way.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <class... KArgs, class... Args>
inline afem_status launch_pdl(afem_context ctx, cudaStream_t s, void (*k)(KArgs...), dim3 grid, unsigned block,
                              Args... args) {
  if (grid.x == 0) return AFEM_OK;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t e = cudaLaunchKernelEx(&cfg, k, static_cast<KArgs>(args)...);
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch (PDL)", __FILE__, __LINE__);
  ++ctx->launches;
  return AFEM_OK;
}

struct GraphChunk {
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  ~GraphChunk() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

// Capture `body(stream)` once into an executable graph.
template <class Body>
inline afem_status capture(afem_context ctx, GraphChunk& g, Body&& body) {
  cudaStream_t cs;
  AFEM_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaStreamDestroy(cs);
    return cuda_fail(e, "cudaStreamBeginCapture", __FILE__, __LINE__);
  }
  int64_t before = ctx->launches;
  afem_status st = body(cs);
  cudaError_t e2 = cudaStreamEndCapture(cs, &g.graph);
  cudaStreamDestroy(cs);
  ctx->launches = before;  // captured kernels are counted when the graph runs
  if (st != AFEM_OK) return st;
  if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture", __FILE__, __LINE__);
  AFEM_CUDA(cudaGraphInstantiate(&g.exec, g.graph, 0));
  return AFEM_OK;
}

// ---------------------------------------------------------------------------
// Sliced-ELL copies of a CSR matrix for the iteration SpMVs (FP64 CG, FCG,
// and the FP32 inner CG of the mixed solver): 32 consecutive rows per slice,
// padded to the slice's longest row; entry k of row 32 s + l sits at
// 32 soff[s] + 32 k + l, so that a warp reads step k of its 32 rows as one
// coalesced 128-byte segment of columns and one of values, where the
// thread-per-row CSR walk reads 32 scattered streams.  Padding entries carry a
// zero weight on the row's own column.  Each row's terms are summed in CSR
// order (a zero weight leaves the sum unchanged), the order of a
// thread-per-row walk of the CSR rows.
constexpr int kSlice = 32;

// slen[s] = the longest row of slice s (one warp per slice)
static __global__ void k_slice_len(int n, const int32_t* __restrict__ rp, int32_t* __restrict__ slen) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nr = ((int64_t)n + kSlice - 1) / kSlice * kSlice;
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < nr; row += stride) {
    const int len = row < n ? __ldg(rp + row + 1) - __ldg(rp + row) : 0;
    const int m = __reduce_max_sync(0xffffffffu, len);
    if ((row & (kSlice - 1)) == 0) slen[row / kSlice] = m;
  }
}

template <class T>
__global__ void k_slice_fill(int n, const int32_t* __restrict__ rp, const int32_t* __restrict__ cols,
                             const double* __restrict__ vals, const int32_t* __restrict__ soff,
                             int32_t* __restrict__ scols, T* __restrict__ svals) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t nr = ((int64_t)n + kSlice - 1) / kSlice * kSlice;
  for (int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; row < nr; row += stride) {
    const int64_t sl = row / kSlice;
    const int m = soff[sl + 1] - soff[sl];
    const int64_t base = (int64_t)kSlice * soff[sl] + (row & (kSlice - 1));
    const int32_t b = row < n ? rp[row] : 0, e = row < n ? rp[row + 1] : 0;
    for (int k = 0; k < m; ++k) {
      const int32_t c = b + k < e ? cols[b + k] : -1;   // -1: past the row, or an unused slot
      const bool in = c >= 0;
      if (scols) scols[base + (int64_t)kSlice * k] = in ? c : (row < n ? (int32_t)row : 0);
      svals[base + (int64_t)kSlice * k] = in ? (T)vals[b + k] : T(0);
    }
  }
}

// Dot product of one sliced row (c, a: the row's first column index and
// value; entries 32 apart) with x, accumulated in Acc in entry order.  Every
// chunk issues all of its loads first (past the row's end they read the
// row's own entry), and the products past the end are skipped by a branch
// that is uniform across the warp (a slice shares its length m), so there is
// neither a serial tail nor a wasted FP64 instruction.
template <class Acc, class T, class V>
__device__ __forceinline__ Acc sliced_row_dot(const int32_t* __restrict__ c, const T* __restrict__ a, int m,
                                              const V* __restrict__ x) {
  Acc acc = Acc(0);
  for (int k = 0; k < m; k += kRowChunk) {
    int32_t cc[kRowChunk];
    T aa[kRowChunk];
#pragma unroll
    for (int u = 0; u < kRowChunk; ++u) {
      const int e = k + u < m ? k + u : 0;
      cc[u] = __ldg(c + (int64_t)kSlice * e);
      aa[u] = __ldg(a + (int64_t)kSlice * e);
    }
#pragma unroll
    for (int u = 0; u < kRowChunk; ++u)
      if (k + u < m) acc = fma((Acc)aa[u], (Acc)__ldg(x + cc[u]), acc);
  }
  return acc;
}

// The copy's device memory (offsets, columns, values), freed stream-ordered
// by release() or the destructor.
template <class T>
struct SlicedCopy {
  cudaStream_t s = nullptr;
  int n = 0;
  int32_t* soff = nullptr;
  int32_t* cols = nullptr;
  T* vals = nullptr;
  void release() {
    if (soff) cudaFreeAsync(soff, s);
    if (cols) cudaFreeAsync(cols, s);
    if (vals) cudaFreeAsync(vals, s);
    soff = cols = nullptr;
    vals = nullptr;
  }
  ~SlicedCopy() { release(); }
};

// scratch of build_slices (slice lengths and the scan's tiles)
inline size_t slices_scratch_bytes(int n) {
  const int64_t nslice = ((int64_t)n + kSlice - 1) / kSlice;
  return align256(sizeof(int32_t) * (size_t)(nslice + 1)) + scan_scratch_bytes(nslice);
}

// Builds the sliced copy of (rp, cols, vals) on the context stream (one
// synchronising read of the copy's size).
template <class T>
afem_status build_slices(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals,
                         SlicedCopy<T>& out) {
  out.release();
  out.s = ctx->stream;
  out.n = n;
  const int64_t nslice = ((int64_t)n + kSlice - 1) / kSlice;
  int32_t* slen;
  AFEM_TRY(scratch_take(ctx, (size_t)nslice + 1, &slen));
  AFEM_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&out.soff), sizeof(int32_t) * (size_t)(nslice + 1), ctx->stream));
  AFEM_TRY(launch(ctx, k_slice_len, grid_for(ctx, nslice * kSlice, 256), 256, 0, n, rp, slen));
  AFEM_TRY(exclusive_scan_i32(ctx, slen, out.soff, nslice));
  int32_t slots = 0;   // sum of the slice lengths (<= nnz); the copy holds 32 x that many entries
  AFEM_TRY(read_scalar(ctx, out.soff + nslice, &slots));
  const size_t entries = (size_t)kSlice * (size_t)std::max(slots, 1);
  AFEM_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&out.cols), sizeof(int32_t) * entries, ctx->stream));
  AFEM_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&out.vals), sizeof(T) * entries, ctx->stream));
  return launch(ctx, k_slice_fill<T>, grid_for(ctx, nslice * kSlice, 256), 256, 0, n, rp, cols, vals,
                (const int32_t*)out.soff, out.cols, out.vals);
}

// Re-reads the values of a matrix whose pattern the copy already holds.
template <class T>
afem_status refill_slice_values(afem_context ctx, const int32_t* rp, const double* vals, const SlicedCopy<T>& sc) {
  const int64_t nslice = ((int64_t)sc.n + kSlice - 1) / kSlice;
  return launch(ctx, k_slice_fill<T>, grid_for(ctx, nslice * kSlice, 256), 256, 0, sc.n, rp,
                (const int32_t*)nullptr, vals, (const int32_t*)sc.soff, (int32_t*)nullptr, sc.vals);
}

// ||b - A x|| / ||b|| in FP64 (rows with skip[i] != 0 left out; skip may be null).
afem_status true_relres(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals,
                        int64_t nnz, const double* b, const double* x, const uint8_t* skip, double* relres);

}  // namespace afem
