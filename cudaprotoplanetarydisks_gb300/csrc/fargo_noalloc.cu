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
// capture.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <mutex>

#include "fargo_device.cuh"
#include "fargo_internal.h"

#define FARGO_NOALLOC_MAX_RINGS 16384
#define FARGO_NOALLOC_MAX_DEVICES 64

// [0, MAX): ring means of Vtheta; [MAX, 2 MAX): per-ring CFL time steps;
// [2 MAX]: the last-block counter (as an unsigned int)
static __device__ __align__(256) double g_noalloc_cfl_scratch[2 * FARGO_NOALLOC_MAX_RINGS + 32];

namespace {

std::mutex g_setup_mutex;
double *g_scratch_addr[FARGO_NOALLOC_MAX_DEVICES] = {nullptr};

// ConditionCFL (src/SourceEuler.cu:520-546, kernels src/Kernels.cu:1267-1359) on
// raw FP64 device arrays; one CTA per ring, the last CTA decides the integer.
__global__ void __launch_bounds__(256) k_cfl_noalloc(const double *__restrict__ vrad, const double *__restrict__ vtheta,
                                                     const double *__restrict__ cs, const double *__restrict__ rinf,
                                                     const double *__restrict__ rmed, const double *__restrict__ rsup,
                                                     int nrad, int nsec, int fast_transport, double deltaT,
                                                     double *scratch, int *cfl_out) {
  __shared__ double s_red[32];
  __shared__ int s_last;
  const int i = blockIdx.x, tid = threadIdx.x;
  double *ring_vmoy = scratch, *ring_newdt = scratch + FARGO_NOALLOC_MAX_RINGS;
  unsigned int *ticket = reinterpret_cast<unsigned int *>(scratch + 2 * FARGO_NOALLOC_MAX_RINGS);
  const double *vth = vtheta + (size_t)i * nsec;
  double s = 0.0;
  for (int j = tid; j < nsec; j += blockDim.x) s += vth[j];
  const double vmoy = block_sum_d(s, s_red) / (double)nsec;
  if (tid == 0) ring_vmoy[i] = vmoy;
  double mn = 1e30;
  if (i > 0) {
    const double dxr = rsup[i] - rinf[i], dxt = rmed[i] * 2.0 * FARGO_PI / (double)nsec;
    const double invdrad = 1.0 / dxr, invdxt = 1.0 / dxt, invmind = 1.0 / ((dxt < dxr) ? dxt : dxr);
    const double *vr = vrad + (size_t)i * nsec, *c = cs + (size_t)i * nsec;
    double mx = 0.0;
    for (int j = tid; j < nsec; j += blockDim.x) {
      const double vres = fast_transport ? vth[j] - vmoy : vth[j];
      const double invdt1 = c[j] * invmind, invdt2 = fabs(vr[j]) * invdrad, invdt3 = fabs(vres) * invdxt;
      double dvr = vr[j + nsec] - vr[j];
      double dvt = vth[j == nsec - 1 ? 0 : j + 1] - vth[j];
      dvr = (dvr >= 0.0) ? 1e-10 : -dvr;
      dvt = (dvt >= 0.0) ? 1e-10 : -dvt;
      const double a4 = dvr * invdrad, b4 = dvt * invdxt;
      double invdt4 = (b4 > a4) ? b4 : a4;
      invdt4 *= 4.0 * FARGO_CVNR * FARGO_CVNR;
      const double S = invdt1 * invdt1 + invdt2 * invdt2 + invdt3 * invdt3 + invdt4 * invdt4;
      mx = (S > mx) ? S : mx;
    }
    mn = FARGO_CFLSECURITY / sqrt(-block_min_d(-mx, s_red));
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
  for (int k = tid; k < nrad - 1; k += blockDim.x) {
    const double v0 = __ldcg(ring_vmoy + k), v1 = __ldcg(ring_vmoy + k + 1);
    m = fmin(m, 2.0 * FARGO_PI * FARGO_CFLSECURITY / (double)nsec / fabs(v0 * (1.0 / rmed[k]) - v1 * (1.0 / rmed[k + 1])));
  }
  m = block_min_d(m, s_red);
  if (tid == 0) {
    if (deltaT < m) m = deltaT;
    const double q = deltaT / m;
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
  k_cfl_noalloc<<<nrad, 256, 0, s>>>(vrad, vtheta, soundspeed, rinf, rmed, rsup, nrad, nsec, fast_transport, deltaT,
                                     scratch, cfl_out);
  return cudaGetLastError() == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}
