// Device characterisation used for rooflines: the FP64 FMA issue rate.
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so the element
// kernels (about 74 FP64 instructions per tetrahedron) are bound by FP64
// issue, not by HBM.  This measures that ceiling on the running device:
// independent FMA chains, every SM busy, timed with CUDA events.
#include "afem_internal.cuh"

namespace afem {

constexpr int kChains = 8;

__global__ void k_dfma_rate(double* out, double a, double b, int iters) {
  double acc[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) acc[c] = threadIdx.x * 1e-3 + c;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) acc[c] = fma(acc[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += acc[c];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace afem

using namespace afem;

extern "C" afem_status afem_device_fp64_fma_rate(afem_context ctx, double* gfma_per_s) {
  AFEM_CHECK_ARG(ctx && gfma_per_s, "afem_device_fp64_fma_rate: bad arguments");
  const int blocks = ctx->sm_count * 8, threads = 256, iters = 2048;
  AFEM_TRY(scratch_reserve(ctx, align256(sizeof(double) * blocks * threads)));
  double* out;
  AFEM_TRY(scratch_take(ctx, (size_t)blocks * threads, &out));
  cudaEvent_t e0, e1;
  AFEM_CUDA(cudaEventCreate(&e0));
  AFEM_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0, ctx->stream);
    afem_status s = launch(ctx, k_dfma_rate, blocks, threads, 0, out, 0.999, 1e-3, iters);
    cudaEventRecord(e1, ctx->stream);
    cudaEventSynchronize(e1);
    if (s != AFEM_OK) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return s;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *gfma_per_s = (double)blocks * threads * iters * kChains / (best * 1e-3) / 1e9;
  return AFEM_OK;
}
