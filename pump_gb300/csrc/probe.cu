// Throughput probe of the binary64 FMA pipe, the roofline denominator of the
// 2pBVP kernels (the measured peaks cover HBM copy and bf16 tensor
// GEMM only).  Eight independent DFMA chains per thread, grid of 8 blocks of
// 256 threads per SM, timed with CUDA events; 2 flops per DFMA.
#include "common.cuh"

namespace pump {
namespace {

__global__ void __launch_bounds__(256) dfma_kernel(int iters, double seed, double *sink) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + threadIdx.x * 1e-9 + k;
  const double m = 0.999999999, c = 1e-12;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], m, c);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 42.0) sink[0] = s;  // keeps the chains live; never true
}

}  // namespace
}  // namespace pump

using namespace pump;

extern "C" pump_status_t pump_probe_fp64_tflops(double *h_tflops, pump_stream_t stream) {
  if (!h_tflops) return set_error(PUMP_ERR_BAD_INPUT, "pump_probe_fp64_tflops: null argument");
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  PUMP_CUDA_TRY(cudaGetDevice(&dev));
  PUMP_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  double *sink = nullptr;
  PUMP_CUDA_TRY(cudaMalloc(&sink, sizeof(double)));
  cudaEvent_t a, b;
  PUMP_CUDA_TRY(cudaEventCreate(&a));
  PUMP_CUDA_TRY(cudaEventCreate(&b));
  const int blocks = sms * 8, threads = 256, iters = 4096;
  dfma_kernel<<<blocks, threads, 0, s>>>(iters / 8, 1.0, sink);  // warm-up
  PUMP_CUDA_TRY(cudaEventRecord(a, s));
  dfma_kernel<<<blocks, threads, 0, s>>>(iters, 1.0, sink);
  PUMP_CUDA_TRY(cudaEventRecord(b, s));
  PUMP_CUDA_TRY(cudaEventSynchronize(b));
  float ms = 0;
  PUMP_CUDA_TRY(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(sink);
  *h_tflops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
  return PUMP_OK;
}
