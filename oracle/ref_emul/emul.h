// emul.h -- TEST INFRASTRUCTURE: CPU execution of the reference's CUDA sources.
//
// Force-included into every reference translation unit built by build_ref.py.
// Kernels become plain functions; a launch runs the grid block by block and, in
// each block, thread by thread in increasing (z, y, x) order -- the launch
// semantics the oracle restates.  Blocks whose kernel calls __syncthreads run
// their threads as cooperative fibers that meet at each barrier.  The CUDA
// runtime calls work on host memory; cuFFT Z2Z calls use the oracle's FFT.
#pragma once
// The reference's global `double *array` (src/Main.cu:39) collides with std::array
// under `using namespace std` (the same clash stops nvcc 13).  The C++ headers the
// reference includes are included here first, and `array` is then renamed for the
// reference's own code only (the last line of this file).
#include <cstdarg>
#include <iostream>
#include <string>
#include <math.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct uint3 {
  unsigned int x, y, z;
};
struct dim3 {
  unsigned int x, y, z;
  dim3(unsigned int a = 1, unsigned int b = 1, unsigned int c = 1) : x(a), y(b), z(c) {}
};
extern thread_local uint3 threadIdx, blockIdx;
extern thread_local dim3 blockDim, gridDim;
#define warpSize 32
#define __global__
#define __device__
#define __host__
#define __shared__
#define __forceinline__ inline
void emu_syncthreads();
#define __syncthreads() emu_syncthreads()

typedef int cudaError_t;
enum { cudaSuccess = 0, cudaErrorInvalidValue = 1, cudaErrorMemoryAllocation = 2 };
enum cudaMemcpyKind {
  cudaMemcpyHostToHost = 0,
  cudaMemcpyHostToDevice = 1,
  cudaMemcpyDeviceToHost = 2,
  cudaMemcpyDeviceToDevice = 3
};
cudaError_t cudaMalloc(void **p, size_t n);
template <class T>
cudaError_t cudaMalloc(T **p, size_t n) {
  return cudaMalloc((void **)p, n);
}
cudaError_t cudaFree(void *p);
cudaError_t cudaMemset(void *p, int v, size_t n);
cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, cudaMemcpyKind k);
cudaError_t cudaDeviceSynchronize();
cudaError_t cudaSetDevice(int d);
const char *cudaGetErrorString(cudaError_t e);
// host min(int, int) that the CUDA headers provide (used by DeviceReduce, src/Kernels.cu:371)
static inline int min(int a, int b) { return a < b ? a : b; }

struct EmuCfg {
  dim3 g, b;
  bool sync;
};
void emu_run(const EmuCfg &c, void (*fn)(void *), void *body);
template <class L>
void emu_trampoline(void *body) {
  (*(L *)body)();
}

template <class F>
struct EmuLauncher {
  F f;
  EmuCfg c;
  template <class... A>
  void operator()(A... args) const {
    auto body = [&]() { f(args...); };
    emu_run(c, &emu_trampoline<decltype(body)>, &body);
  }
};
template <class F>
EmuLauncher<F> emu_make(F f, dim3 g, dim3 b, size_t smem = 0, bool sync = false) {
  (void)smem;
  return EmuLauncher<F>{f, EmuCfg{g, b, sync}};
}

#define array refarray
