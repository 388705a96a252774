// Measured FP64-pipe peak of the current device (fargo_fp64_pipe_peak).
//
// GB300 issues FP64 arithmetic on a narrow pipe (about two lanes per clock per
// SM), and the FP64 mode of the hydro step is bound by it, not by HBM.  Its
// roofline is therefore a measured rate: every thread runs eight independent
// fused-multiply-add chains (enough independent work to cover the FP64 latency),
// 8 CTAs of 256 threads per SM, and the launch is timed with CUDA events after a
// warm-up launch.
#include <cuda_runtime.h>

#include "fargo_gb300.h"

namespace {
constexpr int kChains = 8;
constexpr int kIters = 4096;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_dfma_peak(double *sink, double b, double c) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; k++) x[k] = (double)(threadIdx.x + k) * 1e-3;
  for (int it = 0; it < kIters; it++) {
#pragma unroll
    for (int k = 0; k < kChains; k++) x[k] = fma(x[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; k++) s += x[k];
  if (s == -1.0) sink[0] = s;  // keeps the chains live; never true for these inputs
}
}  // namespace

extern "C" int fargo_fp64_pipe_peak(double *dfma_per_s) {
  if (!dfma_per_s) return FARGO_ERR_INVALID;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FARGO_ERR_CUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return FARGO_ERR_CUDA;
  const int blocks = sms * 8;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return FARGO_ERR_CUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return FARGO_ERR_CUDA;
  }
  float best = 0.f;
  for (int rep = 0; rep < 4; rep++) {  // the first launch warms up; best of the other three
    cudaEventRecord(e0, 0);
    k_dfma_peak<<<blocks, kThreads>>>(nullptr, 0.9999999, 1e-9);
    cudaEventRecord(e1, 0);
    if (cudaEventSynchronize(e1) != cudaSuccess) break;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess || best <= 0.f) return FARGO_ERR_CUDA;
  *dfma_per_s = (double)blocks * kThreads * kIters * kChains / (best * 1e-3);
  return FARGO_OK;
}
