// Measured FP64-pipe peak of the current device (fargo_fp64_pipe_peak), and the
// self-test of the step's FP64 divides (fargo_div_selftest).
//
// GB300 issues FP64 arithmetic on a narrow pipe (about two lanes per clock per
// SM), and the FP64 mode of the hydro step is bound by it, not by HBM.  Its
// roofline is therefore a measured rate: every thread runs eight independent
// fused-multiply-add chains (enough independent work to cover the FP64 latency),
// 8 CTAs of 256 threads per SM, and the launch is timed with CUDA events after a
// warm-up launch.
#include <cuda_runtime.h>

#include "fargo_device.cuh"
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

namespace {
__global__ void k_div_selftest(const double *__restrict__ a, const double *__restrict__ b, int n,
                               double *__restrict__ q_step, double *__restrict__ q_lim) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  q_step[k] = fdiv64(a[k], b[k]);
  q_lim[k] = lim_div(a[k], b[k]);
}
}  // namespace

extern "C" int fargo_div_selftest(const double *a, const double *b, int n, double *q_step, double *q_lim) {
  if (!a || !b || !q_step || !q_lim || n < 1 || n > (1 << 24)) return FARGO_ERR_INVALID;
  double *d = nullptr;
  const size_t bytes = (size_t)n * sizeof(double);
  if (cudaMalloc(&d, 4 * bytes) != cudaSuccess) return FARGO_ERR_CUDA;
  int rc = FARGO_OK;
  if (cudaMemcpy(d, a, bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(d + n, b, bytes, cudaMemcpyHostToDevice) != cudaSuccess)
    rc = FARGO_ERR_CUDA;
  if (rc == FARGO_OK) {
    k_div_selftest<<<(n + 255) / 256, 256>>>(d, d + n, n, d + 2 * (size_t)n, d + 3 * (size_t)n);
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(q_step, d + 2 * (size_t)n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(q_lim, d + 3 * (size_t)n, bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
      rc = FARGO_ERR_CUDA;
  }
  cudaFree(d);
  return rc;
}
