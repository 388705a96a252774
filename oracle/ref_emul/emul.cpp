// emul.cpp -- TEST INFRASTRUCTURE: runtime of the CPU build of the reference (emul.h).
#include <ucontext.h>

#include <cstdlib>
#include <cstring>

#include <cstdint>
#include <vector>

#include "emul.h"
#include "fake_include/cufft.h"
#include "../fft_ref.h"

thread_local uint3 threadIdx, blockIdx;
thread_local dim3 blockDim, gridDim;
double sdata[1 << 16];  // `extern __shared__ double sdata[]` of DeviceReduceKernel

// Every allocation is zero-filled (device memory is zero after allocation in
// practice) and preceded by a zeroed guard: Update_sgvelocityKernel reads
// SG_Acct[(j-1)%nsec] = SG_Acct[-1] at i = j = 0 (src/Kernels.cu:930), and here that
// read sees 0.0, the value the oracle uses, instead of the allocator's bookkeeping.
constexpr size_t kGuard = 256;
cudaError_t cudaMalloc(void **p, size_t n) {
  char *b = static_cast<char *>(std::calloc(kGuard + (n ? n : 1), 1));
  *p = b ? b + kGuard : nullptr;
  return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void *p) {
  if (p) std::free(static_cast<char *>(p) - kGuard);
  return cudaSuccess;
}
cudaError_t cudaMemset(void *p, int v, size_t n) {
  if (!p) return cudaErrorInvalidValue;
  std::memset(p, v, n);
  return cudaSuccess;
}
cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, cudaMemcpyKind) {
  if (!dst || !src) return cudaErrorInvalidValue;  // the runtime rejects null pointers
  std::memmove(dst, src, n);
  return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize() { return cudaSuccess; }
cudaError_t cudaSetDevice(int) { return cudaSuccess; }
const char *cudaGetErrorString(cudaError_t e) {
  switch (e) {
    case cudaSuccess: return "no error";
    case cudaErrorInvalidValue: return "invalid argument";
    case cudaErrorMemoryAllocation: return "out of memory";
  }
  return "unknown error";
}

// ---- grid execution ----------------------------------------------------
namespace {
constexpr size_t kStack = 1 << 16;
struct Fiber {
  ucontext_t ctx;
  char *stack = nullptr;
  uint3 tid;
  bool done = false;
};
ucontext_t g_sched;
Fiber *g_cur = nullptr;
void (*g_fn)(void *) = nullptr;
void *g_bodyp = nullptr;
bool g_fibers = false;

void fiber_entry() {
  g_fn(g_bodyp);
  g_cur->done = true;
  swapcontext(&g_cur->ctx, &g_sched);
}
}  // namespace

void emu_syncthreads() {
  if (!g_fibers) {
    std::fprintf(stderr, "emul: __syncthreads in a kernel launched without barrier support\n");
    std::abort();
  }
  swapcontext(&g_cur->ctx, &g_sched);
}

// Host threads over the blocks of a launch (FARGO_REF_THREADS, default 1), for
// two-dimensional grids only.  No reference kernel but DeviceReduceKernel (run in
// order, below) uses shared memory, barriers or atomics, and every kernel launched
// on a 2D grid guards i < nrad, j < nsec and reads nothing another block of the same
// launch writes, so their blocks' order does not change the result.  The 1D launches
// (boundary kernels over sectors, ring loops) stay in block order: one of them,
// NonReflectingBoundaryKernel2 (src/Kernels.cu:575-589), lets its padded threads
// write into the next ring, and which write lands last depends on that order.
// tests/test_ref_cpu.py checks the one-thread fixtures bitwise on four threads.
int emu_ref_threads() {
  static int n = [] {
    const char *s = std::getenv("FARGO_REF_THREADS");
    const int v = s ? std::atoi(s) : 1;
    return v > 0 ? v : 1;
  }();
  return n;
}

void emu_run(const EmuCfg &c, void (*fn)(void *), void *body) {
  gridDim = c.g;
  blockDim = c.b;
  const unsigned nthr = c.b.x * c.b.y * c.b.z;
  if (!c.sync) {
    const long nblk = (long)c.g.x * c.g.y * c.g.z;
#pragma omp parallel for schedule(static) num_threads(emu_ref_threads()) if (emu_ref_threads() > 1 && c.g.y > 1)
    for (long b = 0; b < nblk; b++) {
      gridDim = c.g;
      blockDim = c.b;
      blockIdx = uint3{(unsigned)(b % c.g.x), (unsigned)((b / c.g.x) % c.g.y), (unsigned)(b / ((long)c.g.x * c.g.y))};
      for (unsigned tz = 0; tz < c.b.z; tz++)
        for (unsigned ty = 0; ty < c.b.y; ty++)
          for (unsigned tx = 0; tx < c.b.x; tx++) {
            threadIdx = uint3{tx, ty, tz};
            fn(body);
          }
    }
    return;
  }
  for (unsigned bz = 0; bz < c.g.z; bz++)
    for (unsigned by = 0; by < c.g.y; by++)
      for (unsigned bx = 0; bx < c.g.x; bx++) {
        blockIdx = uint3{bx, by, bz};
        // cooperative threads: run each until its next barrier, in thread order
        static std::vector<Fiber> pool;  // stacks are allocated once and reused
        if (pool.size() < nthr) pool.resize(nthr);
        g_fn = fn;
        g_bodyp = body;
        g_fibers = true;
        unsigned t = 0;
        for (unsigned tz = 0; tz < c.b.z; tz++)
          for (unsigned ty = 0; ty < c.b.y; ty++)
            for (unsigned tx = 0; tx < c.b.x; tx++, t++) {
              Fiber &f = pool[t];
              f.tid = uint3{tx, ty, tz};
              f.done = false;
              if (!f.stack) f.stack = static_cast<char *>(std::malloc(kStack));
              getcontext(&f.ctx);
              f.ctx.uc_stack.ss_sp = f.stack;
              f.ctx.uc_stack.ss_size = kStack;
              f.ctx.uc_link = nullptr;
              makecontext(&f.ctx, fiber_entry, 0);
            }
        bool all_done = false;
        while (!all_done) {
          all_done = true;
          for (unsigned k = 0; k < nthr; k++) {
            Fiber &f = pool[k];
            if (f.done) continue;
            g_cur = &f;
            threadIdx = f.tid;
            swapcontext(&g_sched, &f.ctx);
            if (!f.done) all_done = false;
          }
        }
        g_fibers = false;
      }
}

// ---- cuFFT Z2Z on the oracle's FFT ----------------------------------------
namespace {
struct Plan {
  int nx, ny;
};
std::vector<Plan> g_plans;
}  // namespace

cufftResult cufftPlan2d(cufftHandle *plan, int nx, int ny, int type) {
  if (type != CUFFT_Z2Z) return CUFFT_INVALID_PLAN;
  g_plans.push_back(Plan{nx, ny});
  *plan = (cufftHandle)g_plans.size();
  return CUFFT_SUCCESS;
}
cufftResult cufftExecZ2Z(cufftHandle plan, cufftDoubleComplex *in, cufftDoubleComplex *out, int direction) {
  if (plan < 1 || plan > (int)g_plans.size()) return CUFFT_INVALID_PLAN;
  const Plan &p = g_plans[plan - 1];
  const size_t n = (size_t)p.nx * p.ny;
  if (out != in) std::memmove(out, in, n * sizeof(cufftDoubleComplex));
  fftref::fft2d(reinterpret_cast<fftref::cplx *>(out), p.nx, p.ny, direction == CUFFT_FORWARD ? -1 : +1);
  return CUFFT_SUCCESS;
}
cufftResult cufftDestroy(cufftHandle) { return CUFFT_SUCCESS; }
