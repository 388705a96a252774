// fargo_force_diag.cu -- the disk's gravitational force on a point, split the way
// the reference's torque diagnostics split it: ComputeForce (src/Force.cu:102-131)
// with ComputeForceKernel (src/Kernels.cu:693-729).
//
// For a point (x, y) with smoothing eps, every cell of mass Surf_i Sigma_ij at
// (Rmed_i cos phi_j, Rmed_i sin phi_j), phi_j = 2 pi j / nsec, pulls with
//   f = G m (dx, dy) / (d^2 + eps^2)^(3/2),
// weighted by the Hill cut 1 - exp(-d^2 / (rh k / (dimfxy - 1))^2) at level k
// (k = 0: no cut), and counts as inner when Rmed_i < a, else outer.  Result: the
// reference's GlobalForce layout, 4 * dimfxy doubles: fx inner [k], fx outer
// [dimfxy + k], fy inner [2 dimfxy + k], fy outer [3 dimfxy + k].
//
// One pass over the grid for all levels (the reference runs dimfxy passes, each
// with four memsets and four reductions): every thread keeps the 44 sums in FP64
// registers over a grid-stride loop; warps and then the CTA reduce them in a fixed
// order, and a second kernel sums the CTA partials in CTA order (deterministic).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "fargo_gb300.h"
#include "fargo_internal.h"

#define FD_LEVELS FARGO_FORCE_LEVELS
#define FD_NSUM (4 * FD_LEVELS)
#define FD_THREADS 128

namespace {

template <class T>
__global__ void __launch_bounds__(FD_THREADS) k_force_partials(const T *__restrict__ dens,
                                                               const double *__restrict__ rmed,
                                                               const double *__restrict__ surf, int nrad, int nsec,
                                                               double x, double y, double eps2, double a, double rh,
                                                               double *__restrict__ part) {
  double acc[FD_NSUM];
#pragma unroll
  for (int k = 0; k < FD_NSUM; k++) acc[k] = 0.0;
  const long long n = (long long)nrad * nsec;
  for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(q / nsec), j = (int)(q - (long long)i * nsec);
    const double cellmass = surf[i] * (double)dens[q];
    const double dx = rmed[i] * cos((2.0 * M_PI * (double)j) / (double)nsec) - x;
    const double dy = rmed[i] * sin((2.0 * M_PI * (double)j) / (double)nsec) - y;
    const double d2 = dx * dx + dy * dy;
    const double dist2 = d2 + eps2;
    const double inv3 = 1.0 / dist2 / sqrt(dist2);
    const double fx = cellmass * dx * inv3, fy = cellmass * dy * inv3;  // G = 1
    const int o = rmed[i] < a ? 0 : FD_LEVELS;
#pragma unroll
    for (int k = 0; k < FD_LEVELS; k++) {
      double cut = 1.0;
      if (k != 0) {
        const double rk = rh * ((double)k / (double)(FD_LEVELS - 1));
        cut = 1.0 - exp(-d2 / (rk * rk));
      }
      // inner and outer sums without a divergent branch: the other half adds 0
      const double wi = o == 0 ? cut : 0.0, wo = o == 0 ? 0.0 : cut;
      acc[k] += fx * wi;
      acc[FD_LEVELS + k] += fx * wo;
      acc[2 * FD_LEVELS + k] += fy * wi;
      acc[3 * FD_LEVELS + k] += fy * wo;
    }
  }
  __shared__ double red[FD_THREADS / 32][FD_NSUM];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
  for (int k = 0; k < FD_NSUM; k++) {
    double v = acc[k];
    for (int s = 16; s > 0; s >>= 1) v += __shfl_down_sync(0xffffffffu, v, s);
    if (lane == 0) red[w][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < FD_NSUM) {
    double v = 0.0;
    for (int ww = 0; ww < FD_THREADS / 32; ww++) v += red[ww][threadIdx.x];
    part[(size_t)blockIdx.x * FD_NSUM + threadIdx.x] = v;
  }
}

__global__ void k_force_final(const double *__restrict__ part, int nparts, double *__restrict__ out) {
  const int k = threadIdx.x;
  if (k >= FD_NSUM) return;
  double v = 0.0;
  for (int b = 0; b < nparts; b++) v += part[(size_t)b * FD_NSUM + k];
  out[k] = v;
}

}  // namespace

extern "C" int fargo_compute_force(fargo_ctx *ctx, double x, double y, double smoothing, double mass, double a,
                                   double rh, double *global_force) {
  (void)mass;  // passed by the reference's ComputeForce, unused by its kernel
  if (!global_force || !(smoothing >= 0.0)) return FARGO_ERR_INVALID;
  DiskView v;
  int rc;
  if ((rc = fargo_disk_view(ctx, &v))) return rc;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev))
    return FARGO_ERR_CUDA;
  const long long n = (long long)v.nrad * v.nsec;
  const int nb = (int)std::min<long long>((long long)sms * 4, (n + FD_THREADS - 1) / FD_THREADS);
  const cudaStream_t s = (cudaStream_t)v.stream;
  double *buf = nullptr;
  if (cudaMallocAsync(&buf, ((size_t)nb + 1) * FD_NSUM * 8, s) != cudaSuccess) return FARGO_ERR_CUDA;
  if (v.esize == 4)
    k_force_partials<float><<<nb, FD_THREADS, 0, s>>>((const float *)v.dens, v.rmed_dev, v.surf_dev, v.nrad, v.nsec,
                                                      x, y, smoothing * smoothing, a, rh, buf + FD_NSUM);
  else
    k_force_partials<double><<<nb, FD_THREADS, 0, s>>>((const double *)v.dens, v.rmed_dev, v.surf_dev, v.nrad,
                                                       v.nsec, x, y, smoothing * smoothing, a, rh, buf + FD_NSUM);
  k_force_final<<<1, 64, 0, s>>>(buf + FD_NSUM, nb, buf);
  cudaError_t e = cudaMemcpyAsync(global_force, buf, FD_NSUM * 8, cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(buf, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}
