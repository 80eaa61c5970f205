// Instrumentation: the sustained FMA rate of the FP64 and FP32 pipes, the
// denominators for the element kernels' compute roofline (the measured peaks
// file covers HBM copy and bf16 tensor throughput only).
#include <cuda_runtime.h>

#include "fq_internal.h"

namespace fq {

template <typename T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T* out, int iters, T a, T b) {
  T x0 = T(threadIdx.x) * T(1e-7), x1 = x0 + T(1), x2 = x0 + T(2), x3 = x0 + T(3);
  T x4 = x0 + T(4), x5 = x0 + T(5), x6 = x0 + T(6), x7 = x0 + T(7);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      x0 = fma(x0, a, b);
      x1 = fma(x1, a, b);
      x2 = fma(x2, a, b);
      x3 = fma(x3, a, b);
      x4 = fma(x4, a, b);
      x5 = fma(x5, a, b);
      x6 = fma(x6, a, b);
      x7 = fma(x7, a, b);
    }
  }
  const T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == T(-12345.678)) out[blockIdx.x] = s;  // keeps the chain alive
}

template <typename T>
static fq_status run_peak(fq_ctx* ctx, double* tflops) {
  int sms = 0;
  FQ_CUDA(ctx, cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device));
  const int blocks = sms * 8, threads = 256;
  const int iters = sizeof(T) == 8 ? 512 : 8192;
  DevBuf out;
  FQ_TRY(out.alloc(ctx, size_t(blocks) * sizeof(T)));
  cudaEvent_t e0, e1;
  FQ_CUDA(ctx, cudaEventCreate(&e0));
  FQ_CUDA(ctx, cudaEventCreate(&e1));
  fma_chain_kernel<T><<<blocks, threads, 0, ctx->stream>>>(out.as<T>(), iters, T(0.999999), T(1e-6));  // warm-up
  FQ_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
  const int reps = 5;
  for (int r = 0; r < reps; ++r)
    fma_chain_kernel<T><<<blocks, threads, 0, ctx->stream>>>(out.as<T>(), iters, T(0.999999), T(1e-6));
  FQ_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
  FQ_CUDA(ctx, cudaEventSynchronize(e1));
  float ms = 0.f;
  FQ_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->launches += reps + 1;
  const double flops = 2.0 * 32.0 * double(iters) * double(blocks) * threads * reps;
  *tflops = flops / (double(ms) * 1e-3) / 1e12;
  return FQ_OK;
}

}  // namespace fq

extern "C" fq_status fq_measure_fma_peak(fq_ctx* ctx, int fp64, double* tflops) {
  if (!ctx || !tflops) return FQ_INVALID_ARG;
  return fp64 ? fq::run_peak<double>(ctx, tflops) : fq::run_peak<float>(ctx, tflops);
}
