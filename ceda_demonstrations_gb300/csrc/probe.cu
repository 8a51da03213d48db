// FP64 issue-rate probe: the denominator the FP64 stage kernel is reported against. Each
// thread runs eight independent FMA chains (enough to cover the FP64 pipe latency) for a
// fixed number of iterations; the grid is a multiple of the SM count. The measured rate is
// 2 flops per FMA over the CUDA-event time of the launch.
#include <cuda_runtime.h>

#include "sts_internal.cuh"

namespace {

constexpr int PROBE_CHAINS = 8;

__global__ void __launch_bounds__(256) fp64_fma_probe_kernel(int iters, double a, double b, double* out)
{
  double v[PROBE_CHAINS];
#pragma unroll
  for (int c = 0; c < PROBE_CHAINS; ++c) v[c] = (double)(threadIdx.x + c) * 1e-3;
  for (int k = 0; k < iters; ++k)
  {
#pragma unroll
    for (int c = 0; c < PROBE_CHAINS; ++c) v[c] = __fma_rn(v[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < PROBE_CHAINS; ++c) s += v[c];
  if (s == 12345.678) out[0] = s; // keeps the chains live; never true for these inputs
}

} // namespace

extern "C" int STS_ProbeFP64Rate(STS_Context ctx, double* tflops)
{
  if (!ctx || !tflops) return STS_ILL_INPUT;
  ctx_activate(ctx);
  const int blocks = ctx->num_sms * 8, threads = 256, iters = 4096;
  double* d = nullptr;
  if (!STS_CUDA_OK(cudaMallocAsync(&d, sizeof(double), ctx->stream))) return STS_ERR_FAILURE;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fp64_fma_probe_kernel<<<blocks, threads, 0, ctx->stream>>>(iters, 0.999999, 1e-7, d); // warm-up
  cudaEventRecord(e0, ctx->stream);
  for (int r = 0; r < 5; ++r) fp64_fma_probe_kernel<<<blocks, threads, 0, ctx->stream>>>(iters, 0.999999, 1e-7, d);
  cudaEventRecord(e1, ctx->stream);
  const bool ok = STS_CUDA_OK(cudaEventSynchronize(e1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(d, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  if (!ok || !(ms > 0.f)) return STS_ERR_FAILURE;
  const double flops = 5.0 * 2.0 * PROBE_CHAINS * (double)iters * blocks * threads;
  *tflops            = flops / (ms * 1e-3) / 1e12;
  return STS_SUCCESS;
}
