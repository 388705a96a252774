// fargo_noalloc.cu -- ConditionCFL for callers that cannot allocate device memory.
//
// Some host programs cannot call cudaMalloc at the point where they need a time
// step: their device memory is owned by another allocator (a framework's caching
// allocator that has reserved the whole device), or they run a latency-critical
// loop where cudaMalloc's implicit device synchronisation would stall their other
// streams.  fargo_condition_cfl_noalloc computes the same CFL integer as
// fargo_condition_cfl from buffers the caller already owns, and keeps its own
// per-ring partial results in a fixed array that is part of the library image.
//
// Limits and sharing: the array holds FARGO_NOALLOC_MAX_RINGS rings; larger grids
// are rejected.  Every GPU that loads the library holds the array until the
// process exits.  All calls share it and it keeps the last call's contents, so
// calls that overlap on the GPU (different streams, or different host threads on
// the same device) race on it.  The first call on each device looks up the array's
// device address with that device current; make that first call before any stream
// capture.  The address is kept for the life of the process: do not use this entry
// point across cudaDeviceReset (or any teardown of the device's primary context).
//
// Arithmetic: the reference's own (see k_cfl_noalloc), so on identical inputs the
// integer is the reference's.  fargo_condition_cfl, the context's fast path, sums
// the ring means as trees and multiplies by per-ring reciprocals; at a rounding tie
// of DeltaT / dt the two can differ by one.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "fargo_device.cuh"
#include "fargo_internal.h"

#define FARGO_NOALLOC_MAX_RINGS 16384
#define FARGO_NOALLOC_MAX_DEVICES 64
#define FARGO_NOALLOC_MAX_SECTORS 16384  // the ring is staged in shared memory (128 KB)

// [0, MAX): ring means of Vtheta; [MAX, 2 MAX): per-ring CFL time steps;
// [2 MAX]: the last-block counter (as an unsigned int)
static __device__ __align__(256) double g_noalloc_cfl_scratch[2 * FARGO_NOALLOC_MAX_RINGS + 32];

namespace {

std::mutex g_setup_mutex;
double *g_scratch_addr[FARGO_NOALLOC_MAX_DEVICES] = {nullptr};

// ConditionCFL (src/SourceEuler.cu:520-546, kernels src/Kernels.cu:1267-1359) on
// raw FP64 device arrays, in the reference's own arithmetic: the ring mean summed
// in j order by one thread (ConditionCFLKernel1D), every per-cell term divided as
// written (ConditionCFLKernel2D1) with no fused multiply-add, the shear limit of
// ConditionCFLKernel2D2 and the final minimum and ceil of ConditionCFLKernel2D3.
// The per-cell time steps are not stored: the ring's minimum of
// CFLSECURITY / sqrt(S) is CFLSECURITY / sqrt(max S), since division and square
// root are correctly rounded and monotone.  One CTA per ring; the last CTA decides.
__global__ void __launch_bounds__(256) k_cfl_noalloc(const double *__restrict__ vrad, const double *__restrict__ vtheta,
                                                     const double *__restrict__ cs, const double *__restrict__ rinf,
                                                     const double *__restrict__ rmed, const double *__restrict__ rsup,
                                                     int nrad, int nsec, int fast_transport, double deltaT,
                                                     double *scratch, int *cfl_out) {
  extern __shared__ double s_ring[];  // the ring's Vtheta, staged for the in-order sum
  __shared__ double s_red[32];
  __shared__ double s_vmoy;
  __shared__ int s_last;
  const int i = blockIdx.x, tid = threadIdx.x;
  double *ring_vmoy = scratch, *ring_newdt = scratch + FARGO_NOALLOC_MAX_RINGS;
  unsigned int *ticket = reinterpret_cast<unsigned int *>(scratch + 2 * FARGO_NOALLOC_MAX_RINGS);
  const double *vth = vtheta + (size_t)i * nsec;
  for (int j = tid; j < nsec; j += blockDim.x) s_ring[j] = vth[j];
  __syncthreads();
  if (tid == 0) {
    double v = 0.0;
    for (int j = 0; j < nsec; j++) v = __dadd_rn(v, s_ring[j]);
    v = __ddiv_rn(v, (double)nsec);
    s_vmoy = v;
    ring_vmoy[i] = v;
  }
  __syncthreads();
  const double vmoy = s_vmoy;
  double mn = 1e30;
  if (i > 0) {
    const double dxrad = __dsub_rn(rsup[i], rinf[i]);
    const double dxtheta = __ddiv_rn(__dmul_rn(__dmul_rn(rmed[i], 2.0), FARGO_PI), (double)nsec);
    const double mind = (dxtheta < dxrad) ? dxtheta : dxrad;  // min2, src/Kernels.cu:1367-1371
    const double *vr = vrad + (size_t)i * nsec, *c = cs + (size_t)i * nsec;
    double mx = 0.0;
    for (int j = tid; j < nsec; j += blockDim.x) {
      const double vres = fast_transport ? __dsub_rn(s_ring[j], vmoy) : s_ring[j];
      const double invdt1 = __ddiv_rn(c[j], mind);
      const double invdt2 = __ddiv_rn(fabs(vr[j]), dxrad);
      const double invdt3 = __ddiv_rn(fabs(vres), dxtheta);
      double dvr = __dsub_rn(vr[j + nsec], vr[j]);
      double dvt = __dsub_rn(s_ring[j == nsec - 1 ? 0 : j + 1], s_ring[j]);
      dvr = (dvr >= 0.0) ? 1e-10 : -dvr;
      dvt = (dvt >= 0.0) ? 1e-10 : -dvt;
      const double a4 = __ddiv_rn(dvr, dxrad), b4 = __ddiv_rn(dvt, dxtheta);
      double invdt4 = (b4 > a4) ? b4 : a4;  // max2, src/Kernels.cu:1361-1365
      invdt4 = __dmul_rn(invdt4, __dmul_rn(__dmul_rn(4.0, FARGO_CVNR), FARGO_CVNR));
      double S = __dmul_rn(invdt1, invdt1);
      S = __dadd_rn(S, __dmul_rn(invdt2, invdt2));
      S = __dadd_rn(S, __dmul_rn(invdt3, invdt3));
      S = __dadd_rn(S, __dmul_rn(invdt4, invdt4));
      mx = (S > mx) ? S : mx;
    }
    mn = __ddiv_rn(FARGO_CFLSECURITY, __dsqrt_rn(-block_min_d(-mx, s_red)));
  }
  if (tid == 0) ring_newdt[i] = mn;
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double m = 1e30;
  for (int k = 1 + tid; k < nrad; k += blockDim.x) m = fmin(m, __ldcg(ring_newdt + k));
  const double num = __ddiv_rn(__dmul_rn(__dmul_rn(2.0, FARGO_PI), FARGO_CFLSECURITY), (double)nsec);
  for (int k = tid; k < nrad - 1; k += blockDim.x) {
    const double v0 = __ldcg(ring_vmoy + k), v1 = __ldcg(ring_vmoy + k + 1);
    const double w = __dsub_rn(__dmul_rn(v0, __ddiv_rn(1.0, rmed[k])), __dmul_rn(v1, __ddiv_rn(1.0, rmed[k + 1])));
    m = fmin(m, __ddiv_rn(num, fabs(w)));
  }
  m = block_min_d(m, s_red);
  if (tid == 0) {
    if (deltaT < m) m = deltaT;
    const double q = __ddiv_rn(deltaT, m);
    *cfl_out = (q > 0.0 && q < 1.0e8) ? (int)ceil(q) : -1;
    *ticket = 0u;
  }
}

}  // namespace

extern "C" int fargo_condition_cfl_noalloc(const double *vrad, const double *vtheta, const double *soundspeed,
                                           const double *rinf, const double *rmed, const double *rsup, int nrad,
                                           int nsec, int fast_transport, double deltaT, void *stream, int *cfl_out) {
  if (!vrad || !vtheta || !soundspeed || !rinf || !rmed || !rsup || !cfl_out || nsec < 4 || nrad < 4 ||
      !(deltaT > 0.0))
    return FARGO_ERR_INVALID;
  if (nsec > FARGO_NOALLOC_MAX_SECTORS) {
    std::fprintf(stderr, "fargo_condition_cfl_noalloc: nsec = %d exceeds the %d sectors a ring's shared staging holds\n",
                 nsec, FARGO_NOALLOC_MAX_SECTORS);
    return FARGO_ERR_INVALID;
  }
  if (nrad > FARGO_NOALLOC_MAX_RINGS) {
    std::fprintf(stderr, "fargo_condition_cfl_noalloc: nrad = %d exceeds the fixed scratch of %d rings\n", nrad,
                 FARGO_NOALLOC_MAX_RINGS);
    return FARGO_ERR_INVALID;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= FARGO_NOALLOC_MAX_DEVICES) return FARGO_ERR_CUDA;
  double *scratch;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
      // one-time set-up on this device: the device address of the static array
      void *p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_cfl_scratch) != cudaSuccess || !p) return FARGO_ERR_CUDA;
      g_scratch_addr[dev] = (double *)p;
    }
    scratch = g_scratch_addr[dev];
  }
  cudaStream_t s = (cudaStream_t)stream;
  // the last-block counter must start at zero; the ring slots are all rewritten
  if (cudaMemsetAsync(scratch + 2 * FARGO_NOALLOC_MAX_RINGS, 0, sizeof(unsigned int), s) != cudaSuccess)
    return FARGO_ERR_CUDA;
  const size_t smem = (size_t)nsec * sizeof(double);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_cfl_noalloc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return FARGO_ERR_CUDA;
  k_cfl_noalloc<<<nrad, 256, smem, s>>>(vrad, vtheta, soundspeed, rinf, rmed, rsup, nrad, nsec, fast_transport,
                                        deltaT, scratch, cfl_out);
  return cudaGetLastError() == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}
