// reduce_wrap.cpp -- TEST INFRASTRUCTURE: DeviceReduce of the CPU build of the
// reference without fibers, linked with -Wl,--wrap on DeviceReduce.
//
// DeviceReduce (src/Kernels.cu:364-394) launches DeviceReduceKernel
// (src/Kernels.cu:253-343) with 32-thread blocks, at most 1024 of them, and sums
// the blocks' partials on the host.  Its five barriers per block make the CPU
// build run every block as 32 cooperative fibers, one context switch per thread
// per barrier, which costs far more than the additions.  This is the same
// arithmetic in the same order, written for one host thread per block:
//  * thread t of block b adds g[i] and g[i + 32] for i = 64 b + t, 64 b + t + 64 nblocks, ...
//    (the second only when i + 32 < N, except for N = 1, where IsPow2's precedence
//    slip (src/Kernels.cu:360) selects the unguarded variant and the read past the
//    single element counts as zero, as in the oracle);
//  * the block's 32 sums fold as s[t] += s[t + 16], s[t + 8], s[t + 4], s[t + 2],
//    s[t + 1] (the pre-sm_30 branch: the CPU build has no __CUDA_ARCH__);
//  * the host adds the blocks' results in block order.
// tests/test_ref_cpu.py checks that the golden fixtures, made with the fiber
// version, are reproduced bitwise.
#include <cstddef>

static long nearest_pow2(long n) {
  if (!n) return n;
  long x = 1;
  while (x < n) x <<= 1;
  return x;
}

int emu_ref_threads();  // emul.cpp: FARGO_REF_THREADS
extern "C" double __real__Z12DeviceReducePdi(double *in, int N);

extern "C" double __wrap__Z12DeviceReducePdi(double *in, int N) {
  const int threads = 32;
  const long nb = (nearest_pow2(N) + threads - 1) / threads;
  const int blocks = nb < 1024 ? (int)nb : 1024;
  const bool pow2 = (N & ((N - 1) == 0)) != 0;
  const unsigned n = (unsigned)N, grid = 2u * threads * (unsigned)blocks;
  double part[1024];
#pragma omp parallel for schedule(static) num_threads(emu_ref_threads()) if (emu_ref_threads() > 1)
  for (int b = 0; b < blocks; b++) {
    double s[threads];
    for (int t = 0; t < threads; t++) {
      unsigned i = (unsigned)b * threads * 2 + t;
      double my = 0.0;
      while (i < n) {
        my += in[i];
        if (pow2 || i + threads < n) my += (i + threads < n) ? in[i + threads] : 0.0;
        i += grid;
      }
      s[t] = my;
    }
    for (int off = 16; off >= 1; off >>= 1)
      for (int t = 0; t < off; t++) s[t] = s[t] + s[t + off];
    part[b] = s[0];
  }
  double sum = 0.0;
  for (int b = 0; b < blocks; b++) sum += part[b];
  return sum;
}
