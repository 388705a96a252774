/*
 * fft_ref.h -- test infrastructure (oracle only; never linked into the product).
 *
 * Unnormalised complex DFT with the cuFFT Z2Z convention the reference calls
 * (cufftPlan2d(2*NRAD, NSEC, CUFFT_Z2Z), src/Main.cu:191-199; cufftExecZ2Z,
 * src/SgMain.cu:117-161):
 *   forward  X[k] = sum_n x[n] exp(-2 pi i k n / N)
 *   inverse  x[n] = sum_k X[k] exp(+2 pi i k n / N)       (no 1/N factor)
 * Recursive mixed-radix decimation in time (any N; small prime factors fast,
 * other factors by direct summation).  cuFFT itself is not under the reference
 * tree (CUDA 13.0 libcufft), so this restatement is pinned against numpy.fft in
 * the CPU tests instead.
 */
#ifndef FFT_REF_H
#define FFT_REF_H

#include <cmath>
#include <complex>
#include <vector>

namespace fftref {

typedef std::complex<double> cplx;

static inline int smallest_factor(int n) {
  for (int p = 2; p * p <= n; ++p)
    if (n % p == 0) return p;
  return n;
}

/* out[0..n) = DFT of in[0], in[stride], ... ; tw[t] = exp(sign 2 pi i t / ntot), t in [0, ntot). */
static void fft_rec(const cplx *in, cplx *out, int n, int stride, const cplx *tw, int ntot,
                    cplx *scratch) {
  if (n == 1) { out[0] = in[0]; return; }
  int p = smallest_factor(n);
  int m = n / p;
  for (int r = 0; r < p; ++r)
    fft_rec(in + (size_t)r * stride, out + (size_t)r * m, m, stride * p, tw, ntot, scratch + n);
  /* butterflies: X[q*m+k] = sum_r W_n^{r (q m + k)} Y_r[k] */
  int step = ntot / n;  /* W_n^t = tw[t*step mod ntot] */
  for (int k = 0; k < m; ++k) {
    for (int q = 0; q < p; ++q) {
      cplx acc(0.0, 0.0);
      int kk = q * m + k;
      for (int r = 0; r < p; ++r) {
        long t = ((long)r * kk) % n;
        acc += out[(size_t)r * m + k] * tw[(size_t)t * step];
      }
      scratch[kk] = acc;
    }
  }
  for (int t = 0; t < n; ++t) out[t] = scratch[t];
}

struct Plan1D {
  int n;
  int sign;
  std::vector<cplx> tw;
  Plan1D(int n_, int sign_) : n(n_), sign(sign_), tw(n_) {
    for (int t = 0; t < n; ++t) {
      double a = 2.0 * M_PI * (double)t / (double)n;
      tw[t] = cplx(std::cos(a), sign * std::sin(a));
    }
  }
  /* in-place transform of x[0], x[stride], ..., x[(n-1)*stride] */
  void exec(cplx *x, int stride, std::vector<cplx> &buf) const {
    buf.resize(4 * (size_t)n + 8);
    cplx *in = buf.data();
    cplx *out = in + n;
    cplx *scr = out + n;
    for (int t = 0; t < n; ++t) in[t] = x[(size_t)t * stride];
    fft_rec(in, out, n, 1, tw.data(), n, scr);
    for (int t = 0; t < n; ++t) x[(size_t)t * stride] = out[t];
  }
};

/* 2D transform of an n0 x n1 row-major array (n1 fastest), like cufftPlan2d(n0, n1). */
static void fft2d(cplx *a, int n0, int n1, int sign) {
  Plan1D p1(n1, sign), p0(n0, sign);
#pragma omp parallel
  {
    std::vector<cplx> buf;
#pragma omp for schedule(static)
    for (int r = 0; r < n0; ++r) p1.exec(a + (size_t)r * n1, 1, buf);
#pragma omp for schedule(static)
    for (int c = 0; c < n1; ++c) p0.exec(a + c, n1, buf);
  }
}

}  // namespace fftref
#endif
