// fargo_learned.cu -- the learned coarse-grid correction around the stencil MLP.
//
// Inputs of the network, per coarse cell (i, j): the 5x5 neighbourhood (rings
// clamped at the edges, sectors periodic) of 5 channels, relative to the centre
// cell so that small perturbations survive BF16: Sigma / Sigma(i, j) - 1 (the
// centre slot: log Sigma(i, j)), the cell-centred v_r, the cell-centred v_theta
// minus the centre's (the centre slot: v_theta minus the Keplerian speed
// r^-1/2), log r minus the centre's (the centre slot: log r), and the azimuth
// from the planet over pi; each of the 125 values normalised by its mean and
// deviation over the training data, padded to 128 (BF16).
//
// Outputs: y_r(i, j), y_phi(i, j), mass-flux corrections through the cell's inner
// radial and left azimuthal interfaces, in units of s * Surf_i (s: the target
// scale).  The density correction is their divergence,
//   dSigma(i, j) = s [y_r(i, j) Surf_i - y_r(i+1, j) Surf_{i+1}] / Surf_i
//                + s [y_phi(i, j) - y_phi(i, j+1)],
// with y_r(0, .) and y_r(nrad, .) taken as zero (walls): the total mass
// sum dSigma Surf telescopes to zero, so the correction conserves mass by
// construction; it is applied only when every density stays positive and the
// rounded mass change stays at roundoff.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "fargo_gb300.h"
#include "fargo_internal.h"

namespace {

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ int wrapj(int j, int n) { return j < 0 ? j + n : (j >= n ? j - n : j); }

struct FeatNorm {
  float mean[125], inv_std[125];
};

// One warp per 32 consecutive cells: each lane forms its cell's 125 inputs in a
// shared row (stride FEAT_LDW words: the lanes' stores of one input fall in
// distinct banks), then the warp writes the 32 rows of 256 bytes out as
// contiguous 128-byte segments.  FP32 arithmetic; the density contrast is
// (Sigma - Sigma_c) / Sigma_c with the difference taken in the field's type.
#define FEAT_LDW 65
template <class T>
__global__ void __launch_bounds__(128) k_features(const T *__restrict__ dens, const T *__restrict__ vrad,
                                                  const T *__restrict__ vtheta, const double *__restrict__ rmed,
                                                  int nrad, int nsec, float phi_planet, FeatNorm nm,
                                                  bf16 *__restrict__ x) {
  __shared__ unsigned srow[4][32 * FEAT_LDW];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n = nrad * nsec, q0 = (blockIdx.x * 4 + w) * 32;
  if (q0 >= n) return;  // whole warps
  const int q = q0 + lane;
  bf16 *row = reinterpret_cast<bf16 *>(&srow[w][lane * FEAT_LDW]);
  if (q < n) {
    const int i = q / nsec, j = q - (q / nsec) * nsec;
    const float dphi = 6.28318530717958648f / (float)nsec;
    const size_t c0 = (size_t)i * nsec + j;
    const T d0 = dens[c0];
    const float inv_d0 = 1.0f / (float)d0;
    const float vt0 = 0.5f * ((float)vtheta[c0] + (float)vtheta[(size_t)i * nsec + wrapj(j + 1, nsec)]);
    const float lr0 = logf((float)rmed[i]);
#pragma unroll
    for (int di = -2; di <= 2; di++) {
      const int ii = min(max(i + di, 0), nrad - 1);
      const float r = (float)rmed[ii];
      const float lr = di == 0 ? lr0 : logf(r) - lr0;
#pragma unroll
      for (int dj = -2; dj <= 2; dj++) {
        const int jj = wrapj(j + dj, nsec), jp = wrapj(jj + 1, nsec);
        const size_t c = (size_t)ii * nsec + jj;
        float ang = (jj + 0.5f) * dphi - phi_planet;  // cell centre azimuth relative to the planet
        ang -= 6.28318530717958648f * floorf(ang * 0.15915494309189535f + 0.5f);
        float v[5];
        if (di == 0 && dj == 0) {
          v[0] = logf((float)d0);
          v[2] = vt0 - rsqrtf(r);
          v[3] = lr0;
        } else {
          v[0] = (float)(dens[c] - d0) * inv_d0;
          v[2] = 0.5f * ((float)vtheta[c] + (float)vtheta[(size_t)ii * nsec + jp]) - vt0;
          v[3] = di == 0 ? 0.0f : lr;
        }
        v[1] = 0.5f * ((float)vrad[c] + (float)vrad[c + nsec]);
        v[4] = ang * 0.31830988618379067f;
        const int base = ((di + 2) * 5 + (dj + 2)) * 5;
#pragma unroll
        for (int ch = 0; ch < 5; ch++)
          row[base + ch] = __float2bfloat16_rn((v[ch] - nm.mean[base + ch]) * nm.inv_std[base + ch]);
      }
    }
    row[125] = row[126] = row[127] = __float2bfloat16_rn(0.0f);
  }
  __syncwarp();
  for (int r = 0; r < 32 && q0 + r < n; r++) {
    unsigned *dst = reinterpret_cast<unsigned *>(x + (size_t)(q0 + r) * 128);
    dst[lane] = srow[w][r * FEAT_LDW + lane];
    dst[lane + 32] = srow[w][r * FEAT_LDW + lane + 32];
  }
}

// dSigma of the flux corrections (see the file comment)
__global__ void k_divergence(const float *__restrict__ y, const double *__restrict__ surf, int nrad, int nsec,
                             float scale, float *__restrict__ ds) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nrad * nsec) return;
  const int i = q / nsec, j = q % nsec;
  const float yr0 = i > 0 ? y[(size_t)q * 2] : 0.0f;
  const float yr1 = i + 1 < nrad ? y[((size_t)q + nsec) * 2] : 0.0f;
  const float yp0 = y[(size_t)q * 2 + 1], yp1 = y[((size_t)i * nsec + wrapj(j + 1, nsec)) * 2 + 1];
  const float s1 = i + 1 < nrad ? (float)(surf[i + 1] / surf[i]) : 0.0f;
  ds[q] = scale * ((yr0 - yr1 * s1) + (yp0 - yp1));
}

// Positivity limiter of the correction (donor-cell limiting in the manner of
// flux-corrected transport, Zalesak 1979).  In mass units the correction moves
// s y_r(i, j) Surf_i through the inner face of (i, j) (into the cell when
// positive) and s y_phi(i, j) Surf_i through its left face.  R(i, j) = the
// fraction of its outflows a cell can afford: min(1, beta Sigma Surf_i / outflow).
// Every face flux is then scaled by the R of its donor cell, so no cell loses more
// than beta of its mass and each face keeps one flux for both cells (the total
// mass is conserved as before).
template <class T>
__global__ void k_limit_ratio(const float *__restrict__ y, const T *__restrict__ dens,
                              const double *__restrict__ surf, int nrad, int nsec, float scale, float beta,
                              float *__restrict__ R) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nrad * nsec) return;
  const int i = q / nsec, j = q % nsec;
  const double s = scale, Si = surf[i];
  double out = 0.0;
  if (i > 0) out += fmax(0.0, -s * y[(size_t)q * 2] * Si);
  if (i + 1 < nrad) out += fmax(0.0, s * y[((size_t)q + nsec) * 2] * surf[i + 1]);
  out += fmax(0.0, -s * y[(size_t)q * 2 + 1] * Si);
  out += fmax(0.0, s * y[((size_t)i * nsec + wrapj(j + 1, nsec)) * 2 + 1] * Si);
  const double avail = (double)beta * (double)dens[q] * Si;
  R[q] = out > avail ? (float)(avail / out) : 1.0f;
}

// dSigma of the limited face fluxes
__global__ void k_divergence_limited(const float *__restrict__ y, const double *__restrict__ surf,
                                     const float *__restrict__ R, int nrad, int nsec, float scale,
                                     float *__restrict__ ds) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nrad * nsec) return;
  const int i = q / nsec, j = q % nsec;
  const int jl = wrapj(j - 1, nsec), jr = wrapj(j + 1, nsec);
  const double s = scale, Si = surf[i];
  double fin = 0.0, fout = 0.0;
  if (i > 0) {  // into (i, j) through its inner face; donor (i - 1, j) when positive
    const double F = s * y[(size_t)q * 2] * Si;
    fin = F * (F < 0.0 ? R[q] : R[q - nsec]);
  }
  if (i + 1 < nrad) {  // out of (i, j) through its outer face; donor (i, j) when positive
    const double F = s * y[((size_t)q + nsec) * 2] * surf[i + 1];
    fout = F * (F > 0.0 ? R[q] : R[q + nsec]);
  }
  const double G = s * y[(size_t)q * 2 + 1] * Si;  // into (i, j) from (i, j - 1)
  const double gin = G * (G < 0.0 ? R[q] : R[(size_t)i * nsec + jl]);
  const double H = s * y[((size_t)i * nsec + jr) * 2 + 1] * Si;  // out of (i, j) into (i, j + 1)
  const double gout = H * (H > 0.0 ? R[q] : R[(size_t)i * nsec + jr]);
  ds[q] = (float)((fin - fout + gin - gout) / Si);
}

// Ring-neutral projection of the radial outputs: y_r(i, .) minus its mean over
// the ring (FP64 sum in a fixed order), in place.  Applied to y before the
// divergence, every ring's mass change sum_j dSigma Surf_i vanishes, so the
// azimuthally averaged density is the plain step's; the projection is symmetric,
// so applied to dL/dy_r it is also its own adjoint.
__global__ void k_ring_center(float *__restrict__ y2, int nsec) {
  __shared__ double red[256];
  const int i = blockIdx.x, tid = threadIdx.x;
  float *row = y2 + (size_t)i * nsec * 2;
  double sum = 0.0;
  for (int j = tid; j < nsec; j += blockDim.x) sum += (double)row[(size_t)j * 2];
  red[tid] = sum;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (tid < w) red[tid] += red[tid + w];
    __syncthreads();
  }
  const float mean = (float)(red[0] / (double)nsec);
  for (int j = tid; j < nsec; j += blockDim.x) row[(size_t)j * 2] -= mean;
}

// e = 2 (dSigma - target) / (n var); per-block sums of (dSigma - target)^2
__global__ void k_residual(const float *__restrict__ ds, const float *__restrict__ target, int n, float e_scale,
                           float *__restrict__ e, double *__restrict__ part) {
  __shared__ double red[256];
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  double sq = 0.0;
  if (q < n) {
    const float d = ds[q] - target[q];
    e[q] = e_scale * d;
    sq = (double)d * d;
  }
  red[threadIdx.x] = sq;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_sum_parts(const double *__restrict__ part, int n, double *__restrict__ out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < n; k++) s += part[k];
    *out = s;
  }
}

// dL/dy from dL/dSigma = e (the adjoint of k_divergence)
__global__ void k_adjoint(const float *__restrict__ e, const double *__restrict__ surf, int nrad, int nsec,
                          float scale, float *__restrict__ dy) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nrad * nsec) return;
  const int i = q / nsec, j = q % nsec;
  float gr = 0.0f;
  if (i > 0) gr = scale * (e[q] - e[q - nsec] * (float)(surf[i] / surf[i - 1]));
  const float gp = scale * (e[q] - e[(size_t)i * nsec + wrapj(j - 1, nsec)]);
  dy[(size_t)q * 2] = gr;
  dy[(size_t)q * 2 + 1] = gp;
}

// fine -> coarse restriction by a factor F: area-weighted density, interface
// velocities averaged over the fine interfaces that make up the coarse one
template <class T>
__global__ void k_restrict(const T *__restrict__ fd, const T *__restrict__ fvr, const T *__restrict__ fvt,
                           const double *__restrict__ fsurf, int F, int cnrad, int cnsec,
                           double *__restrict__ cd, double *__restrict__ cvr, double *__restrict__ cvt) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (cnrad + 1) * cnsec) return;
  const int i = q / cnsec, j = q % cnsec, fnsec = F * cnsec;
  // interface velocity: the fine interface F i, over the F sectors of coarse sector j
  double vr = 0.0;
  for (int b = 0; b < F; b++) vr += (double)fvr[(size_t)(F * i) * fnsec + F * j + b];
  cvr[q] = vr / F;
  if (i == cnrad) {  // ghost ring: density and azimuthal velocity of the fine ghost ring
    double d = 0.0, vt = 0.0;
    for (int b = 0; b < F; b++) {
      d += (double)fd[(size_t)(F * i) * fnsec + F * j + b];
      vt += (double)fvt[(size_t)(F * i) * fnsec + F * j + b];
    }
    cd[q] = d / F;
    cvt[q] = vt / F;
    return;
  }
  double m = 0.0, a = 0.0, vt = 0.0;
  for (int ai = 0; ai < F; ai++) {
    const int fi = F * i + ai;
    const double sf = fsurf[fi];
    for (int b = 0; b < F; b++) m += (double)fd[(size_t)fi * fnsec + F * j + b] * sf;
    a += F * sf;
    // azimuthal face F j of the fine ring, weighted by the ring's surface
    vt += (double)fvt[(size_t)fi * fnsec + F * j] * sf;
  }
  cd[q] = m / a;
  cvt[q] = vt / (a / F);
}

// candidate density and per-ring checks: non-positive or non-finite cells,
// sum dSigma Surf and sum |dSigma| Surf
template <class T>
__global__ void k_apply_check(const T *__restrict__ dens, const float *__restrict__ ds, const double *__restrict__ surf,
                              int nsec, T *__restrict__ cand, double *__restrict__ ring) {
  __shared__ double r0[256], r1[256];
  __shared__ int bad;
  const int i = blockIdx.x;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  double s0 = 0.0, s1 = 0.0;
  for (int j = threadIdx.x; j < nsec; j += blockDim.x) {
    const size_t q = (size_t)i * nsec + j;
    const T v = dens[q] + (T)ds[q];
    cand[q] = v;
    if (!(v > (T)0) || !isfinite((double)v)) atomicOr(&bad, 1);
    s0 += (double)ds[q];
    s1 += fabs((double)ds[q]);
  }
  r0[threadIdx.x] = s0;
  r1[threadIdx.x] = s1;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      r0[threadIdx.x] += r0[threadIdx.x + o];
      r1[threadIdx.x] += r1[threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    ring[3 * i] = r0[0] * surf[i];
    ring[3 * i + 1] = r1[0] * surf[i];
    ring[3 * i + 2] = bad;
  }
}

template <class T>
__global__ void k_density_out(const T *__restrict__ d, int n, float *__restrict__ out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < n) out[q] = (float)d[q];
}
}  // namespace

extern "C" {

int fargo_learned_features(int esize, const void *dens, const void *vrad, const void *vtheta, const double *rmed,
                           int nrad, int nsec, double phi_planet, const float *norm, void *x, void *stream) {
  if ((esize != 4 && esize != 8) || !dens || !vrad || !vtheta || !rmed || !norm || !x || nrad < 1 || nsec < 1)
    return FARGO_ERR_INVALID;
  FeatNorm nm;
  for (int c = 0; c < 125; c++) {
    nm.mean[c] = norm[c];
    nm.inv_std[c] = norm[125 + c] > 0.0f ? 1.0f / norm[125 + c] : 1.0f;
  }
  const int n = nrad * nsec;
  const cudaStream_t s = (cudaStream_t)stream;
  const int nb = (n + 127) / 128;  // 4 warps of 32 cells
  if (esize == 4)
    k_features<float><<<nb, 128, 0, s>>>((const float *)dens, (const float *)vrad, (const float *)vtheta, rmed, nrad,
                                         nsec, (float)phi_planet, nm, (bf16 *)x);
  else
    k_features<double><<<nb, 128, 0, s>>>((const double *)dens, (const double *)vrad, (const double *)vtheta, rmed,
                                          nrad, nsec, (float)phi_planet, nm, (bf16 *)x);
  return cudaGetLastError() == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

int fargo_learned_divergence_limited(fargo_ctx *ctx, const float *y, float scale, float beta, float *ds) {
  if (!y || !ds || !(beta > 0.0f && beta < 1.0f)) return FARGO_ERR_INVALID;
  DiskView v;
  int rc;
  if ((rc = fargo_disk_view(ctx, &v))) return rc;
  const int n = v.nrad * v.nsec, nb = (n + 255) / 256;
  const cudaStream_t s = (cudaStream_t)v.stream;
  float *R = (float *)v.cand;  // scratch: the candidate density of fargo_learned_apply comes later
  if (v.esize == 4)
    k_limit_ratio<float><<<nb, 256, 0, s>>>(y, (const float *)v.dens, v.surf_dev, v.nrad, v.nsec, scale, beta, R);
  else
    k_limit_ratio<double><<<nb, 256, 0, s>>>(y, (const double *)v.dens, v.surf_dev, v.nrad, v.nsec, scale, beta, R);
  k_divergence_limited<<<nb, 256, 0, s>>>(y, v.surf_dev, R, v.nrad, v.nsec, scale, ds);
  if (cudaGetLastError() != cudaSuccess) return FARGO_ERR_CUDA;
  return cudaStreamSynchronize(s) == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

int fargo_learned_ring_center(float *y, int nrad, int nsec, void *stream) {
  if (!y || nrad < 1 || nsec < 1) return FARGO_ERR_INVALID;
  k_ring_center<<<nrad, 256, 0, (cudaStream_t)stream>>>(y, nsec);
  return cudaGetLastError() == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

int fargo_learned_divergence(const float *y, const double *surf, int nrad, int nsec, float scale, float *ds,
                             void *stream) {
  if (!y || !surf || !ds || nrad < 1 || nsec < 1) return FARGO_ERR_INVALID;
  const int n = nrad * nsec;
  k_divergence<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(y, surf, nrad, nsec, scale, ds);
  return cudaGetLastError() == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

// *loss (device) = sum (dSigma - target)^2; e and dy for L = that sum * inv_var / n
int fargo_learned_loss(const float *y, const float *target, const double *surf, int nrad, int nsec, float scale,
                       float inv_var, float *ds, float *e, float *dy, double *part, double *loss, void *stream) {
  if (!y || !target || !surf || !ds || !e || !dy || !part || !loss || nrad < 1 || nsec < 1) return FARGO_ERR_INVALID;
  const int n = nrad * nsec, nb = (n + 255) / 256;
  const cudaStream_t s = (cudaStream_t)stream;
  k_divergence<<<nb, 256, 0, s>>>(y, surf, nrad, nsec, scale, ds);
  k_residual<<<nb, 256, 0, s>>>(ds, target, n, 2.0f * inv_var / (float)n, e, part);
  k_sum_parts<<<1, 32, 0, s>>>(part, nb, loss);
  k_adjoint<<<nb, 256, 0, s>>>(e, surf, nrad, nsec, scale, dy);
  return cudaGetLastError() == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

// Sets the coarse disk's density and velocities to the restriction of the fine
// disk's (fine grid = factor x the coarse one in both directions, same extent).
int fargo_learned_restrict(fargo_ctx *fine, fargo_ctx *coarse, int factor) {
  DiskView f, c;
  int rc;
  if ((rc = fargo_disk_view(fine, &f)) || (rc = fargo_disk_view(coarse, &c))) return rc;
  if (factor < 1 || f.nrad != factor * c.nrad || f.nsec != factor * c.nsec || f.esize != c.esize)
    return FARGO_ERR_INVALID;
  const size_t nc = (size_t)(c.nrad + 1) * c.nsec;
  const double *fsurf = f.surf_dev;
  double *buf = nullptr;
  if (cudaMalloc(&buf, 3 * nc * 8) != cudaSuccess) return FARGO_ERR_CUDA;
  const int nb = (int)((nc + 255) / 256);
  const cudaStream_t s = (cudaStream_t)f.stream;
  if (f.esize == 4)
    k_restrict<float><<<nb, 256, 0, s>>>((const float *)f.dens, (const float *)f.vrad, (const float *)f.vtheta, fsurf,
                                         factor, c.nrad, c.nsec, buf, buf + nc, buf + 2 * nc);
  else
    k_restrict<double><<<nb, 256, 0, s>>>((const double *)f.dens, (const double *)f.vrad, (const double *)f.vtheta,
                                          fsurf, factor, c.nrad, c.nsec, buf, buf + nc, buf + 2 * nc);
  std::vector<double> h(3 * nc);
  cudaError_t e = cudaMemcpyAsync(h.data(), buf, 3 * nc * 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(buf);
  if (e != cudaSuccess) return FARGO_ERR_CUDA;
  return fargo_set_fields(coarse, h.data(), h.data() + nc, h.data() + 2 * nc, nullptr);
}

int fargo_learned_features_ctx(fargo_ctx *ctx, const float *norm, void *x) {
  DiskView v;
  int rc;
  if (!norm || !x) return FARGO_ERR_INVALID;
  if ((rc = fargo_disk_view(ctx, &v))) return rc;
  rc = fargo_learned_features(v.esize, v.dens, v.vrad, v.vtheta, v.rmed_dev, v.nrad, v.nsec, v.planet_phi, norm, x,
                              v.stream);
  const cudaError_t e = cudaStreamSynchronize((cudaStream_t)v.stream);
  return rc ? rc : (e == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA);
}

int fargo_learned_density(fargo_ctx *ctx, float *out) {
  DiskView v;
  int rc;
  if (!out) return FARGO_ERR_INVALID;
  if ((rc = fargo_disk_view(ctx, &v))) return rc;
  const int n = v.nrad * v.nsec;
  const cudaStream_t s = (cudaStream_t)v.stream;
  if (v.esize == 4) k_density_out<float><<<(n + 255) / 256, 256, 0, s>>>((const float *)v.dens, n, out);
  else k_density_out<double><<<(n + 255) / 256, 256, 0, s>>>((const double *)v.dens, n, out);
  return cudaStreamSynchronize(s) == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

// Adds the correction ds (device float, nrad * nsec) to the disk's density when
// every cell stays positive and |sum ds Surf| <= 1e-5 sum |ds| Surf (+1e-300);
// *accepted = 1 then, else 0 and the density is unchanged.  *dmass: sum ds Surf.
int fargo_learned_apply(fargo_ctx *ctx, const float *ds, int *accepted, double *dmass) {
  DiskView v;
  int rc;
  if (!ds || !accepted) return FARGO_ERR_INVALID;
  *accepted = 0;
  if ((rc = fargo_disk_view(ctx, &v))) return rc;
  const size_t n = (size_t)v.nrad * v.nsec;
  const double *surf = v.surf_dev;
  double *ring = v.ring;
  void *cand = v.cand;
  cudaError_t e = cudaSuccess;
  const cudaStream_t s = (cudaStream_t)v.stream;
  std::vector<double> h(3 * (size_t)v.nrad);
  if (e == cudaSuccess) {
    if (v.esize == 4)
      k_apply_check<float><<<v.nrad, 256, 0, s>>>((const float *)v.dens, ds, surf, v.nsec, (float *)cand, ring);
    else
      k_apply_check<double><<<v.nrad, 256, 0, s>>>((const double *)v.dens, ds, surf, v.nsec, (double *)cand, ring);
    e = cudaMemcpyAsync(h.data(), ring, h.size() * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e == cudaSuccess) {
    double dm = 0.0, am = 0.0;
    bool bad = false;
    for (int i = 0; i < v.nrad; i++) {
      dm += h[3 * i];
      am += h[3 * i + 1];
      bad = bad || h[3 * i + 2] != 0.0;
    }
    if (dmass) *dmass = dm;
    if (!bad && std::fabs(dm) <= 1e-5 * am + 1e-300) {
      e = cudaMemcpyAsync(v.dens, cand, n * v.esize, cudaMemcpyDeviceToDevice, s);
      if (e == cudaSuccess) e = cudaStreamSynchronize(s);
      if (e == cudaSuccess) *accepted = 1;
    }
  }
  return e == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA;
}

}  // extern "C"
