// fargo_sg.cu -- self-gravity as a hand-written FFT convolution in log r.
//
// Restates compute_selfgravity (src/SgMain.cu:23-45) and its kernels
// ComputeFFTKernel / ComputeConvolutionKernel / ComputeSgAccKernel
// (src/Kernels.cu:840-912).  The reference zero-pads the radial direction to
// 2*NRAD, runs four forward and two inverse complex cuFFT Z2Z transforms of the
// 2*NRAD x NSEC grid per call, and recomputes the constant kernel spectra every
// time.  Here:
//   * the kernel spectra K^r, K^theta are transformed once at set-up;
//   * the two real fields S_r, S_theta of a ring share one complex FFT along the
//     azimuth (z = S_r + i S_theta), and only the NSEC/2+1 non-redundant modes
//     are kept (real input => Hermitian spectrum);
//   * the radial transform of each mode skips the zero half of the padding;
//   * the inverse runs the same way backwards, and the two real accelerations
//     come out of one inverse FFT per ring.
// Every FFT is a radix-4/2/3 Stockham transform in shared memory, FP64 in both
// precision modes (the convolution accumulation stays FP64).
#include <cuda_runtime.h>

#include "fargo_device.cuh"
#include "fargo_kernels.cuh"

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }

// Forward Stockham FFT of length N on shared buffers d0 -> (d0|d1); returns the
// buffer holding the result.  tw[t] = exp(-2 pi i t / N).
__device__ double2 *fft_fwd(double2 *d0, double2 *d1, int N, const int *rad, int nst, const double2 *__restrict__ tw) {
  int Ns = 1;
  for (int s = 0; s < nst; s++) {
    const int R = rad[s], NR = N / R, tws = N / (Ns * R);
    for (int j = threadIdx.x; j < NR; j += blockDim.x) {
      const int jj = j % Ns;
      double2 v[4];
#pragma unroll
      for (int r = 0; r < 4; r++) {
        if (r < R) {
          v[r] = d0[j + r * NR];
          if (r > 0) v[r] = cmul(v[r], __ldg(tw + r * jj * tws));
        }
      }
      if (R == 2) {
        double2 a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
      } else if (R == 4) {
        double2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
        double2 s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
        v[0] = cadd(s02, s13);
        v[2] = csub(s02, s13);
        v[1] = make_double2(d02.x + d13.y, d02.y - d13.x);  // d02 - i d13
        v[3] = make_double2(d02.x - d13.y, d02.y + d13.x);  // d02 + i d13
      } else {  // R == 3
        const double h = 0.86602540378443864676;  // sqrt(3)/2
        double2 t1 = cadd(v[1], v[2]);
        double2 t2 = make_double2(v[0].x - 0.5 * t1.x, v[0].y - 0.5 * t1.y);
        double2 t3 = csub(v[1], v[2]);
        v[0] = cadd(v[0], t1);
        v[1] = make_double2(t2.x + h * t3.y, t2.y - h * t3.x);  // t2 - i h t3
        v[2] = make_double2(t2.x - h * t3.y, t2.y + h * t3.x);  // t2 + i h t3
      }
      const int idxD = (j / Ns) * Ns * R + jj;
#pragma unroll
      for (int r = 0; r < 4; r++)
        if (r < R) d1[idxD + r * Ns] = v[r];
    }
    __syncthreads();
    double2 *t = d0;
    d0 = d1;
    d1 = t;
    Ns *= R;
  }
  return d0;
}

}  // namespace

int sg_radices(int n, int *rad) {
  int k = 0;
  while (n % 4 == 0) { rad[k++] = 4; n /= 4; }
  while (n % 2 == 0) { rad[k++] = 2; n /= 2; }
  while (n % 3 == 0) { rad[k++] = 3; n /= 3; }
  if (n != 1 || k > 16) return -1;
  return k;
}

// Azimuthal forward transform of rows [0, nrows): ComputeFFTKernel packing
// (S_r = Sigma sqrt(r/r0), S_theta = S_r r/r0, src/Kernels.cu:858-861) when
// src == 0, the real kernel tables (set-up) when src == 1.  Output: modes
// m < M of each real field, stored column-major [m][row] with leading dimension ld.
template <class T>
__global__ void __launch_bounds__(256) k_sg_rows_fwd(KArgs<T> a, int src, double2 *out_r, double2 *out_t, int ld) {
  extern __shared__ __align__(16) double2 sg_smem[];
  const int i = blockIdx.x, nsec = a.P.nsec;
  double2 *b0 = sg_smem, *b1 = sg_smem + nsec;
  if (src == 0) {
    const double f = RT64(a, RT_SGSQRT, i), rm = RT64(a, RT_RMED, i), r0 = RT64(a, RT_RMED, 0);
    for (int j = threadIdx.x; j < nsec; j += blockDim.x) {
      const double var = (double)a.d.dens[(size_t)i * nsec + j] * f;
      b0[j] = make_double2(var, var * rm / r0);
    }
  } else {
    for (int j = threadIdx.x; j < nsec; j += blockDim.x)
      b0[j] = make_double2(a.sg.kr[(size_t)i * nsec + j], a.sg.kt[(size_t)i * nsec + j]);
  }
  __syncthreads();
  double2 *Z = fft_fwd(b0, b1, nsec, a.sg.rad1, a.sg.nst1, a.sg.tw1);
  for (int m = threadIdx.x; m < a.sg.M; m += blockDim.x) {
    const double2 z = Z[m], zc = cconj(Z[m == 0 ? 0 : nsec - m]);
    // X_r = (Z[m] + conj Z[N-m]) / 2, X_t = (Z[m] - conj Z[N-m]) / (2i)
    const double2 xr = make_double2(0.5 * (z.x + zc.x), 0.5 * (z.y + zc.y));
    const double2 d = csub(z, zc);
    const double2 xt = make_double2(0.5 * d.y, -0.5 * d.x);
    out_r[(size_t)m * ld + i] = xr;
    out_t[(size_t)m * ld + i] = xt;
  }
}

// Radial transforms, one CTA per azimuthal mode m.  mode 1 (set-up): forward
// transform of the kernel spectra columns in place.  mode 0: for (S_r, K^r) and
// (S_theta, K^theta): forward transform of the zero-padded column, product
// -G K^ S^ (ComputeConvolutionKernel src/Kernels.cu:871-890), inverse transform,
// rows < nrad stored back in place.
template <class T>
__global__ void __launch_bounds__(256) k_sg_cols(KArgs<T> a, int mode) {
  extern __shared__ __align__(16) double2 sg_smem[];
  const int m = blockIdx.x, n0 = 2 * a.P.nrad, nrad = a.P.nrad;
  double2 *b0 = sg_smem, *b1 = sg_smem + n0;
  for (int f = 0; f < 2; f++) {
    double2 *kh = (f == 0 ? a.sg.khat_r : a.sg.khat_t) + (size_t)m * n0;
    if (mode == 1) {
      for (int k = threadIdx.x; k < n0; k += blockDim.x) b0[k] = kh[k];
      __syncthreads();
      double2 *X = fft_fwd(b0, b1, n0, a.sg.rad0, a.sg.nst0, a.sg.tw0);
      for (int k = threadIdx.x; k < n0; k += blockDim.x) kh[k] = X[k];
      __syncthreads();
      continue;
    }
    double2 *col = (f == 0 ? a.sg.spec_r : a.sg.spec_t) + (size_t)m * nrad;
    for (int k = threadIdx.x; k < n0; k += blockDim.x) b0[k] = (k < nrad) ? col[k] : make_double2(0.0, 0.0);
    __syncthreads();
    double2 *X = fft_fwd(b0, b1, n0, a.sg.rad0, a.sg.nst0, a.sg.tw0);
    double2 *Y = (X == b0) ? b1 : b0;
    for (int k = threadIdx.x; k < n0; k += blockDim.x) {
      const double2 K = kh[k], S = X[k];
      // -G*(K S); stored conjugated so that the forward routine runs the inverse
      const double gx = -1.0 * (K.x * S.x - K.y * S.y);
      const double gy = -1.0 * (K.x * S.y + K.y * S.x);
      Y[k] = make_double2(gx, -gy);
    }
    __syncthreads();
    double2 *Z = fft_fwd(Y, X, n0, a.sg.rad0, a.sg.nst0, a.sg.tw0);
    for (int k = threadIdx.x; k < nrad; k += blockDim.x) col[k] = cconj(Z[k]);
    __syncthreads();
  }
}

// Inverse azimuthal transform of each ring + ComputeSgAccKernel (src/Kernels.cu:893-912).
template <class T>
__global__ void __launch_bounds__(256) k_sg_rows_inv(KArgs<T> a) {
  extern __shared__ __align__(16) double2 sg_smem[];
  const int i = blockIdx.x, nsec = a.P.nsec, nrad = a.P.nrad, M = a.sg.M;
  double2 *b0 = sg_smem, *b1 = sg_smem + nsec;
  for (int m = threadIdx.x; m < nsec; m += blockDim.x) {
    double2 hr, ht;
    if (m < M) {
      hr = a.sg.spec_r[(size_t)m * nrad + i];
      ht = a.sg.spec_t[(size_t)m * nrad + i];
    } else {
      hr = cconj(a.sg.spec_r[(size_t)(nsec - m) * nrad + i]);
      ht = cconj(a.sg.spec_t[(size_t)(nsec - m) * nrad + i]);
    }
    // Z = H_r + i H_t, conjugated for the inverse
    b0[m] = make_double2(hr.x - ht.y, -(hr.y + ht.x));
  }
  __syncthreads();
  double2 *Z = fft_fwd(b0, b1, nsec, a.sg.rad1, a.sg.nst1, a.sg.tw1);
  const double normr = RT64(a, RT_SGNORMR, i), normt = RT64(a, RT_SGNORMT, i);
  const double selfc = a.P.sgp_rstep, tstep = a.P.sgp_tstep, eps = a.P.sgp_eps;
  for (int j = threadIdx.x; j < nsec; j += blockDim.x) {
    const double2 z = cconj(Z[j]);
    const size_t q = (size_t)i * nsec + j;
    a.d.sg_acct[q] = (T)(z.y * normt);
    double accr = z.x * normr;
    accr += 1.0 * (double)a.d.dens[q] * selfc * tstep / eps;
    a.d.sg_accr[q] = (T)accr;
  }
}

template <class T>
void launch_selfgravity(const KArgs<T> &a, cudaStream_t s) {
  const int nsec = a.P.nsec, nrad = a.P.nrad;
  k_sg_rows_fwd<T><<<nrad, 256, 2 * nsec * sizeof(double2), s>>>(a, 0, a.sg.spec_r, a.sg.spec_t, nrad);
  probe_mark(s, "k_sg_rows_fwd");
  k_sg_cols<T><<<a.sg.M, 256, 2 * 2 * nrad * sizeof(double2), s>>>(a, 0);
  probe_mark(s, "k_sg_cols");
  k_sg_rows_inv<T><<<nrad, 256, 2 * nsec * sizeof(double2), s>>>(a);
  probe_mark(s, "k_sg_rows_inv");
}

// Set-up: spectra of the constant kernels (compute_kernel src/SgMain.cu:49-81 is
// evaluated on the host; its transforms are done once here).
template <class T>
void launch_sg_kernel_spectra(const KArgs<T> &a, cudaStream_t s) {
  const int nsec = a.P.nsec, n0 = 2 * a.P.nrad;
  k_sg_rows_fwd<T><<<n0, 256, 2 * nsec * sizeof(double2), s>>>(a, 1, a.sg.khat_r, a.sg.khat_t, n0);
  k_sg_cols<T><<<a.sg.M, 256, 2 * n0 * sizeof(double2), s>>>(a, 1);
}

template <class T>
cudaError_t prepare_sg_kernels(int nsec, int n0) {
  cudaError_t e;
  int rows = (int)(2 * nsec * sizeof(double2)), cols = (int)(2 * n0 * sizeof(double2));
  if ((e = cudaFuncSetAttribute(k_sg_rows_fwd<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, rows)) != cudaSuccess) return e;
  if ((e = cudaFuncSetAttribute(k_sg_rows_inv<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, rows)) != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_sg_cols<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, cols);
}

#define INSTANTIATE_SG(T)                                                      \
  template void launch_selfgravity<T>(const KArgs<T> &, cudaStream_t);         \
  template void launch_sg_kernel_spectra<T>(const KArgs<T> &, cudaStream_t);   \
  template cudaError_t prepare_sg_kernels<T>(int, int);
INSTANTIATE_SG(double)
INSTANTIATE_SG(float)
