// Shared pieces of the Krylov solvers (CG, mixed-precision CG, flexible CG
// with the learned preconditioner): G-lanes-per-row CSR dot products,
// deterministic last-block reductions, the lanes-per-row choice, and CUDA
// graph capture of a chunk of iterations.
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
      const bool in = k + u < e;
      c[u] = in ? __ldg(cols + k + u) : row;
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
  for (int32_t k = __ldg(rp + row) + lane; k < e; k += G) s += (double)__ldg(vals + k) * (double)__ldg(x + __ldg(cols + k));
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

// ||b - A x|| / ||b|| in FP64 (rows with skip[i] != 0 left out; skip may be null).
afem_status true_relres(afem_context ctx, int n, const int32_t* rp, const int32_t* cols, const double* vals,
                        int64_t nnz, const double* b, const double* x, const uint8_t* skip, double* relres);

}  // namespace afem
