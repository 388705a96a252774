// fargo_sg.cu -- self-gravity as a hand-written FFT convolution in log r.
//
// Restates compute_selfgravity (src/SgMain.cu:23-45) and its kernels
// ComputeFFTKernel / ComputeConvolutionKernel / ComputeSgAccKernel
// (src/Kernels.cu:840-912).  The reference zero-pads the radial direction to
// 2*NRAD, runs four forward and two inverse complex cuFFT Z2Z transforms of the
// 2*NRAD x NSEC grid per call, and recomputes the constant kernel spectra every
// time.  Here:
//   * the kernel spectra K^r, K^theta are transformed once at set-up, in FP64;
//   * the two real fields S_r, S_theta of a ring share one complex FFT along the
//     azimuth (z = S_r + i S_theta), and only the NSEC/2+1 non-redundant modes
//     are kept (real input => Hermitian spectrum);
//   * the radial transform of each mode skips the zero half of the padding;
//   * the inverse runs the same way backwards, and the two real accelerations
//     come out of one inverse FFT per ring.
// Every FFT is a radix-4/2/3 Stockham transform in shared memory.  The per-step
// transforms run in the field type: FP64 in the FP64 mode; FP32 in the FP32-bulk
// mode (complex float, kernel spectra rounded from their FP64 set-up), where an
// FP64 FFT would run on a pipe 64 times narrower than the FP32 one.
#include <cuda_runtime.h>

#include <initializer_list>

#include "fargo_device.cuh"
#include "fargo_kernels.cuh"

namespace {

template <class R>
struct Vec2;
template <>
struct Vec2<double> {
  using t = double2;
};
template <>
struct Vec2<float> {
  using t = float2;
};

__device__ __forceinline__ double2 mk2(double x, double y) { return make_double2(x, y); }
__device__ __forceinline__ float2 mk2(float x, float y) { return make_float2(x, y); }
template <class V>
__device__ __forceinline__ V cmul(V a, V b) {
  return mk2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <class V>
__device__ __forceinline__ V cadd(V a, V b) {
  return mk2(a.x + b.x, a.y + b.y);
}
template <class V>
__device__ __forceinline__ V csub(V a, V b) {
  return mk2(a.x - b.x, a.y - b.y);
}
template <class V>
__device__ __forceinline__ V cconj(V a) {
  return mk2(a.x, -a.y);
}

// Shared-memory FFT buffers hold element i at fpad(i) = i + i/8: the stride-8
// stores of a radix-8 stage then spread over the banks instead of hitting two.
__host__ __device__ __forceinline__ int fpad(int i) { return i + (i >> 3); }
__host__ __device__ __forceinline__ int fpadn(int n) { return n + (n >> 3) + 1; }

// DFT of length RAD in registers (forward, exp(-2 pi i / RAD)).
template <int RAD, class V>
__device__ __forceinline__ void butterfly(V *v) {
  using R = decltype(v[0].x);
  if (RAD == 2) {
    const V a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  } else if (RAD == 3) {
    const R h = (R)0.86602540378443864676;  // sqrt(3)/2
    const V t1 = cadd(v[1], v[2]);
    const V t2 = mk2(v[0].x - (R)0.5 * t1.x, v[0].y - (R)0.5 * t1.y);
    const V t3 = csub(v[1], v[2]);
    v[0] = cadd(v[0], t1);
    v[1] = mk2(t2.x + h * t3.y, t2.y - h * t3.x);  // t2 - i h t3
    v[2] = mk2(t2.x - h * t3.y, t2.y + h * t3.x);  // t2 + i h t3
  } else if (RAD == 4) {
    const V s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    const V s13 = cadd(v[1], v[3]), d13 = csub(v[1], v[3]);
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = mk2(d02.x + d13.y, d02.y - d13.x);  // d02 - i d13
    v[3] = mk2(d02.x - d13.y, d02.y + d13.x);  // d02 + i d13
  } else {  // RAD == 8: two DFT4 of the even and odd points, then W8^k
    V e[4] = {v[0], v[2], v[4], v[6]}, o[4] = {v[1], v[3], v[5], v[7]};
    butterfly<4>(e);
    butterfly<4>(o);
    const R h = (R)0.70710678118654752440;  // 1/sqrt(2)
    const V w1 = mk2((o[1].x + o[1].y) * h, (o[1].y - o[1].x) * h);    // (1 - i)/sqrt2 o1
    const V w2 = mk2(o[2].y, -o[2].x);                                  // -i o2
    const V w3 = mk2((o[3].y - o[3].x) * h, -(o[3].y + o[3].x) * h);   // -(1 + i)/sqrt2 o3
    v[0] = cadd(e[0], o[0]);
    v[4] = csub(e[0], o[0]);
    v[1] = cadd(e[1], w1);
    v[5] = csub(e[1], w1);
    v[2] = cadd(e[2], w2);
    v[6] = csub(e[2], w2);
    v[3] = cadd(e[3], w3);
    v[7] = csub(e[3], w3);
  }
}

// One Stockham stage of radix RAD over src (length N, Ns = product of the
// earlier radices): butterflies j = lt, lt + G, ...; out(index, value) stores.
template <int RAD, class V, class Out>
__device__ __forceinline__ void fft_stage(const V *src, int N, int Ns, const V *tw, int lt, int G, Out out) {
  const int NR = N / RAD, tws = N / (Ns * RAD);
  // Ns is a power of two in every stage before a radix-3 one (radices run 8, 4,
  // 2, then 3): shift and mask instead of integer division there
  const bool p2 = (Ns & (Ns - 1)) == 0;
  const int lg = __ffs(Ns) - 1;
  for (int j = lt; j < NR; j += G) {
    const int jj = p2 ? (j & (Ns - 1)) : j % Ns;
    const int jb = p2 ? (j >> lg) : j / Ns;
    V v[RAD];
#pragma unroll
    for (int r = 0; r < RAD; r++) {
      v[r] = src[fpad(j + r * NR)];
      if (r > 0) v[r] = cmul(v[r], tw[r * jj * tws]);
    }
    butterfly<RAD>(v);
    const int idxD = jb * Ns * RAD + jj;
#pragma unroll
    for (int r = 0; r < RAD; r++) out(idxD + r * Ns, v[r]);
  }
}

// Forward Stockham FFT of length N from d0, ping-ponging with d1, by the G
// threads lt = 0..G-1 of a group (every thread of the CTA calls it: one barrier
// per stage).  tw[t] = exp(-2 pi i t / N).  The last stage hands its outputs to
// last(index, value, free buffer); the default stores them there.  Returns the
// buffer the last stage wrote to when last stores into the free buffer.
template <class V, class Last>
__device__ V *fft_run(V *d0, V *d1, int N, const int *rad, int nst, const V *tw, int lt, int G, Last last) {
  int Ns = 1;
  for (int s = 0; s < nst; s++) {
    const int R = rad[s];
    V *dst = d1;
    if (s == nst - 1) {
      auto out = [&](int k, V v) { last(k, v, dst); };
      if (R == 8) fft_stage<8>(d0, N, Ns, tw, lt, G, out);
      else if (R == 4) fft_stage<4>(d0, N, Ns, tw, lt, G, out);
      else if (R == 2) fft_stage<2>(d0, N, Ns, tw, lt, G, out);
      else fft_stage<3>(d0, N, Ns, tw, lt, G, out);
    } else {
      auto out = [&](int k, V v) { dst[fpad(k)] = v; };
      if (R == 8) fft_stage<8>(d0, N, Ns, tw, lt, G, out);
      else if (R == 4) fft_stage<4>(d0, N, Ns, tw, lt, G, out);
      else if (R == 2) fft_stage<2>(d0, N, Ns, tw, lt, G, out);
      else fft_stage<3>(d0, N, Ns, tw, lt, G, out);
    }
    __syncthreads();
    V *t = d0;
    d0 = d1;
    d1 = t;
    Ns *= R;
  }
  return d0;
}

template <class V>
struct StoreFree {
  __device__ __forceinline__ void operator()(int k, V v, V *dst) const { dst[fpad(k)] = v; }
};

// Compile-time plans for the common lengths: the radices in the order
// sg_radices gives (8s, then 4s, 2s, 3s), every stage's stride, butterfly count
// and buffer offsets constants, so that a stage is its loads, butterflies and
// stores.  Same arithmetic as fft_run (a stage with Ns = 1 skips the unit
// twiddle, which changes no finite value).
__host__ __device__ constexpr int plan_radix_of(int n) { return n % 8 == 0 ? 8 : n % 4 == 0 ? 4 : n % 2 == 0 ? 2 : 3; }
__host__ __device__ constexpr int plan_nst(int n) {
  int k = 0;
  while (n > 1) {
    n /= plan_radix_of(n);
    k++;
  }
  return k;
}
__host__ __device__ constexpr int plan_rad(int n, int s) {
  for (int k = 0; k < s; k++) n /= plan_radix_of(n);
  return plan_radix_of(n);
}
__host__ __device__ constexpr int plan_ns(int n, int s) {
  int ns = 1;
  for (int k = 0; k < s; k++) {
    const int r = plan_radix_of(n);
    ns *= r;
    n /= r;
  }
  return ns;
}

// Twiddles of a stage: read from the shared table ...
template <class V>
struct TwShared {
  const V *tw;
  template <int S, int TWS>
  __device__ __forceinline__ V get(int r, int jj) const {
    return tw[r * jj * TWS];
  }
};
// ... or held in registers, when every stage has at most one butterfly per
// thread (N / radix <= G): a thread needs radix - 1 twiddles per stage, loaded
// once from the global table and used by every transform of the kernel.
template <int N>
__host__ __device__ constexpr bool plan_fits(int g) {
  for (int s = 0; s < plan_nst(N); s++)
    if (N / plan_rad(N, s) > g) return false;
  return true;
}
template <int N, class V>
struct TwRegs {
  V w[plan_nst(N)][7];
  template <int S, int TWS>
  __device__ __forceinline__ V get(int r, int) const {
    return w[S][r - 1];
  }
};
template <int N, int S, class V>
__device__ __forceinline__ void tw_regs_load(TwRegs<N, V> &t, const V *twg, int lt) {
  constexpr int R = plan_rad(N, S), NS = plan_ns(N, S), NR = N / R, TWS = N / (NS * R);
  if constexpr (NS > 1) {
    const int jj = (lt < NR ? lt : 0) % NS;
#pragma unroll
    for (int r = 1; r < R; r++) t.w[S][r - 1] = twg[r * jj * TWS];
  }
  if constexpr (S + 1 < plan_nst(N)) tw_regs_load<N, S + 1>(t, twg, lt);
}

template <int N, int S, int RAD, int NS, int G, class V, class Tw, class Out>
__device__ __forceinline__ void fft_stage_c(const V *src, const Tw &tw, int lt, Out out) {
  constexpr int NR = N / RAD, TWS = N / (NS * RAD);
#pragma unroll
  for (int k = 0; k < (NR + G - 1) / G; k++) {
    const int j = lt + k * G;
    if (NR % G == 0 || j < NR) {
      const int jj = j % NS, jb = j / NS;
      V v[RAD];
#pragma unroll
      for (int r = 0; r < RAD; r++) {
        v[r] = src[fpad(j + r * NR)];
        if (r > 0 && NS > 1) v[r] = cmul(v[r], tw.template get<S, TWS>(r, jj));
      }
      butterfly<RAD>(v);
      const int idxD = jb * NS * RAD + jj;
#pragma unroll
      for (int r = 0; r < RAD; r++) out(idxD + r * NS, v[r]);
    }
  }
}

template <int N, int S, int G, class V, class Tw, class Last>
__device__ __forceinline__ V *fft_run_c(V *d0, V *d1, const Tw &tw, int lt, Last last) {
  constexpr int R = plan_rad(N, S), NS = plan_ns(N, S), NST = plan_nst(N);
  if constexpr (S == NST - 1) {
    fft_stage_c<N, S, R, NS, G>(d0, tw, lt, [&](int k, V v) { last(k, v, d1); });
    __syncthreads();
    return d1;
  } else {
    fft_stage_c<N, S, R, NS, G>(d0, tw, lt, [&](int k, V v) { d1[fpad(k)] = v; });
    __syncthreads();
    return fft_run_c<N, S + 1, G>(d1, d0, tw, lt, last);
  }
}

// The compile-time plan for N > 0, the run-time one (rad, nst) for N = 0.
template <int N, int G, class V, class Last>
__device__ __forceinline__ V *fft_any(V *d0, V *d1, int n, const int *rad, int nst, const V *tw, int lt, Last last) {
  if constexpr (N > 0) return fft_run_c<N, 0, G>(d0, d1, TwShared<V>{tw}, lt, last);
  else return fft_run(d0, d1, n, rad, nst, tw, lt, G, last);
}

// Splits the FFT Z of two packed real rows into the modes m < M of each:
// X_r = (Z[m] + conj Z[N-m]) / 2, X_t = (Z[m] - conj Z[N-m]) / (2i)
template <class V>
__device__ __forceinline__ void unpack_pair(const V *Z, int m, int N, V &xr, V &xt) {
  const V z = Z[fpad(m)], zc = cconj(Z[fpad(m == 0 ? 0 : N - m)]);
  xr = mk2((decltype(z.x))0.5 * (z.x + zc.x), (decltype(z.x))0.5 * (z.y + zc.y));
  const V d = csub(z, zc);
  xt = mk2((decltype(z.x))0.5 * d.y, (decltype(z.x))-0.5 * d.x);
}

}  // namespace

int sg_radices(int n, int *rad) {
  int k = 0;
  while (n % 8 == 0 && k < 16) { rad[k++] = 8; n /= 8; }
  while (n % 4 == 0 && k < 16) { rad[k++] = 4; n /= 4; }
  while (n % 2 == 0 && k < 16) { rad[k++] = 2; n /= 2; }
  while (n % 3 == 0 && k < 16) { rad[k++] = 3; n /= 3; }
  if (n != 1) return -1;
  return k;
}

// threads per FFT group for length n: one radix-8 butterfly per thread and stage
__host__ __device__ constexpr int sg_group(int n) {
  return (n / 8 + 31) / 32 * 32 < 32 ? 32 : ((n / 8 + 31) / 32 * 32 > 256 ? 256 : (n / 8 + 31) / 32 * 32);
}
// threads per field group of the radial kernel (two groups per CTA)
__host__ __device__ constexpr int sg_col_group(int n0) { return sg_group(n0) < 128 ? sg_group(n0) : 128; }

// Azimuthal forward transform of each ring with the ComputeFFTKernel packing
// (S_r = Sigma sqrt(r/r0), S_theta = S_r r/r0, src/Kernels.cu:858-861).  Output:
// modes m < M of each real field, column-major [m][ring].
template <class T, int NSEC>
__global__ void __launch_bounds__(256) k_sg_rows_fwd(KArgs<T> a) {
  pdl_enter();
  if (a.guard && a.d.ctl->done) return;  // the next substep's, after the DT's last
  using V = typename Vec2<T>::t;
  extern __shared__ __align__(16) unsigned char sg_raw[];
  constexpr int G = 256;
  const int i = blockIdx.x, nsec = NSEC > 0 ? NSEC : a.P.nsec, nrad = a.P.nrad, tid = threadIdx.x;
  V *tw = (V *)sg_raw, *b0 = tw + nsec, *b1 = b0 + fpadn(nsec);
  const V *twg = (const V *)a.sg.tw1;
  const T f = RT(a, RT_SGSQRT, i), rm = RT(a, RT_RMED, i), r0 = RT(a, RT_RMED, 0);
#pragma unroll 4
  for (int j = tid; j < nsec; j += G) {
    tw[j] = twg[j];
    const T var = a.d.dens[(size_t)i * nsec + j] * f;
    b0[fpad(j)] = mk2(var, var * rm / r0);
  }
  __syncthreads();
  V *Z = fft_any<NSEC, G>(b0, b1, nsec, a.sg.rad1, a.sg.nst1, tw, tid, StoreFree<V>());
  V *out_r = (V *)a.sg.spec_r, *out_t = (V *)a.sg.spec_t;
  for (int m = tid; m < a.sg.M; m += G) {
    V xr, xt;
    unpack_pair(Z, m, nsec, xr, xt);
    out_r[(size_t)m * nrad + i] = xr;
    out_t[(size_t)m * nrad + i] = xt;
  }
}

// Radial transforms, one CTA per azimuthal mode m, one thread group per field:
// (S_r, K^r) and (S_theta, K^theta) side by side.  Forward transform of the
// zero-padded column; its last stage forms -G K^ S^ (ComputeConvolutionKernel
// src/Kernels.cu:871-890), conjugated so that the forward routine runs the
// inverse; the inverse's last stage stores rows < nrad ring-major (the
// scattered side of the transpose is a store here, a contiguous load after).
template <class T, int N0>
__global__ void __launch_bounds__(256) k_sg_cols(KArgs<T> a) {
  pdl_enter();
  if (a.guard && a.d.ctl->done) return;  // the next substep's, after the DT's last
  using V = typename Vec2<T>::t;
  extern __shared__ __align__(16) unsigned char sg_raw[];
  constexpr int GC = N0 > 0 ? sg_col_group(N0) : 0;
  const int m = blockIdx.x, n0 = N0 > 0 ? N0 : 2 * a.P.nrad, nrad = n0 >> 1;
  const int G = N0 > 0 ? GC : (int)(blockDim.x >> 1), g = threadIdx.x >= G ? 1 : 0, lt = threadIdx.x - g * G;
  V *tw = (V *)sg_raw;
  V *b0 = tw + n0 + g * 3 * fpadn(n0), *b1 = b0 + fpadn(n0), *K = b1 + fpadn(n0);
  const V *twg = (const V *)a.sg.tw0;
  const V *kh = (const V *)(g == 0 ? a.sg.khat_r : a.sg.khat_t) + (size_t)m * n0;
  V *col = (V *)(g == 0 ? a.sg.spec_r : a.sg.spec_t) + (size_t)m * nrad;
  V *row = (V *)(g == 0 ? a.sg.spec2_r : a.sg.spec2_t) + m;  // ring-major output, stride M
  // twiddles in registers when the plan allows it, else in shared memory
  constexpr bool REG = N0 > 0 && plan_fits<(N0 > 0 ? N0 : 2)>(GC);
  TwRegs<(N0 > 0 ? N0 : 2), V> tr;
  if constexpr (REG) {
    tw_regs_load<N0, 0>(tr, twg, lt);
  } else {
#pragma unroll 4
    for (int k = threadIdx.x; k < n0; k += blockDim.x) tw[k] = twg[k];
  }
#pragma unroll 4
  for (int k = lt; k < n0; k += G) {
    K[fpad(k)] = kh[k];
    b0[fpad(k)] = (k < nrad) ? col[k] : mk2((T)0, (T)0);
  }
  __syncthreads();
  auto conv = [&](int k, V S, V *dst) {
    const V Kk = K[fpad(k)];
    const T gx = (T)-1.0 * (Kk.x * S.x - Kk.y * S.y);
    const T gy = (T)-1.0 * (Kk.x * S.y + Kk.y * S.x);
    dst[fpad(k)] = mk2(gx, -gy);
  };
  auto store = [&](int k, V z, V *) {
    if (k < nrad) row[(size_t)k * a.sg.M] = cconj(z);
  };
  if constexpr (REG) {
    V *X = fft_run_c<N0, 0, GC>(b0, b1, tr, lt, conv);
    fft_run_c<N0, 0, GC>(X, (X == b0) ? b1 : b0, tr, lt, store);
  } else if constexpr (N0 > 0) {
    V *X = fft_run_c<N0, 0, GC>(b0, b1, TwShared<V>{tw}, lt, conv);
    fft_run_c<N0, 0, GC>(X, (X == b0) ? b1 : b0, TwShared<V>{tw}, lt, store);
  } else {
    V *X = fft_run(b0, b1, n0, a.sg.rad0, a.sg.nst0, tw, lt, G, conv);
    fft_run(X, (X == b0) ? b1 : b0, n0, a.sg.rad0, a.sg.nst0, tw, lt, G, store);
  }
}

// Inverse azimuthal transform of each ring; its last stage applies
// ComputeSgAccKernel (src/Kernels.cu:893-912).
template <class T, int NSEC>
__global__ void __launch_bounds__(256) k_sg_rows_inv(KArgs<T> a) {
  pdl_enter();
  if (a.guard && a.d.ctl->done) return;  // the next substep's, after the DT's last
  using V = typename Vec2<T>::t;
  extern __shared__ __align__(16) unsigned char sg_raw[];
  constexpr int G = 256;
  const int i = blockIdx.x, nsec = NSEC > 0 ? NSEC : a.P.nsec, M = NSEC > 0 ? NSEC / 2 + 1 : a.sg.M, tid = threadIdx.x;
  V *tw = (V *)sg_raw, *b0 = tw + nsec, *b1 = b0 + fpadn(nsec);
  T *dn = (T *)(b1 + fpadn(nsec));  // the ring's density, for the epilogue
  const V *twg = (const V *)a.sg.tw1;
  const size_t row = (size_t)i * nsec;
  const T normr = RT(a, RT_SGNORMR, i), normt = RT(a, RT_SGNORMT, i);
  // this ring's row of the ring-major spectra that k_sg_cols left
  const V *spr = (const V *)a.sg.spec2_r + (size_t)i * M, *spt = (const V *)a.sg.spec2_t + (size_t)i * M;
#pragma unroll 4
  for (int m = tid; m < nsec; m += G) {
    tw[m] = twg[m];
    dn[m] = a.d.dens[row + m];
    V hr, ht;
    if (m < M) {
      hr = spr[m];
      ht = spt[m];
    } else {
      hr = cconj(spr[nsec - m]);
      ht = cconj(spt[nsec - m]);
    }
    // Z = H_r + i H_t, conjugated for the inverse
    b0[fpad(m)] = mk2(hr.x - ht.y, -(hr.y + ht.x));
  }
  __syncthreads();
  const T selfc = (T)a.P.sgp_rstep, tstep = (T)a.P.sgp_tstep, eps = (T)a.P.sgp_eps, sgself = KC(T, a, KC_SGSELF);
  fft_any<NSEC, G>(b0, b1, nsec, a.sg.rad1, a.sg.nst1, tw, tid, [&](int j, V v, V *) {
    const V z = cconj(v);
    const size_t q = row + j;
    a.d.sg_acct[q] = z.y * normt;
    T accr = z.x * normr;
    // FP64: the reference's expression; FP32: its constant factor folded once
    accr += sizeof(T) == 8 ? (T)1.0 * dn[j] * selfc * tstep / eps : dn[j] * sgself;
    a.d.sg_accr[q] = accr;
  });
}

// dynamic shared memory of k_sg_rows_inv: twiddles, two FFT buffers, the density
template <class T>
static size_t sg_rows_inv_smem(int nsec) {
  return (nsec + 2 * fpadn(nsec)) * 2 * sizeof(T) + nsec * sizeof(T);
}

// Kernel instance for a length: the compile-time plan when the length has one.
template <class T>
using SgKernel = void (*)(KArgs<T>);
template <class T>
SgKernel<T> sg_rows_fwd_fn(int nsec) {
  switch (nsec) {
    case 384: return k_sg_rows_fwd<T, 384>;
    case 512: return k_sg_rows_fwd<T, 512>;
    case 768: return k_sg_rows_fwd<T, 768>;
    case 1024: return k_sg_rows_fwd<T, 1024>;
    case 1536: return k_sg_rows_fwd<T, 1536>;
    default: return k_sg_rows_fwd<T, 0>;
  }
}
template <class T>
SgKernel<T> sg_rows_inv_fn(int nsec) {
  switch (nsec) {
    case 384: return k_sg_rows_inv<T, 384>;
    case 512: return k_sg_rows_inv<T, 512>;
    case 768: return k_sg_rows_inv<T, 768>;
    case 1024: return k_sg_rows_inv<T, 1024>;
    case 1536: return k_sg_rows_inv<T, 1536>;
    default: return k_sg_rows_inv<T, 0>;
  }
}
template <class T>
SgKernel<T> sg_cols_fn(int n0) {
  switch (n0) {
    case 256: return k_sg_cols<T, 256>;
    case 512: return k_sg_cols<T, 512>;
    case 1024: return k_sg_cols<T, 1024>;
    case 2048: return k_sg_cols<T, 2048>;
    default: return k_sg_cols<T, 0>;
  }
}

// The azimuthal forward transforms of the rings (they read only the density).
template <class T>
void launch_sg_rows_fwd(const KArgs<T> &a, cudaStream_t s) {
  const int nsec = a.P.nsec, nrad = a.P.nrad;
  const size_t vs = 2 * sizeof(T);
  launch_k(a.pdl, sg_rows_fwd_fn<T>(a.sg_generic ? 0 : nsec), dim3(nrad), dim3(256), (nsec + 2 * fpadn(nsec)) * vs, s, a);
  probe_mark(s, "k_sg_rows_fwd");
}

// The radial convolution and the inverse azimuthal transforms (accelerations).
template <class T>
void launch_sg_cols_inv(const KArgs<T> &a, cudaStream_t s) {
  const int nsec = a.P.nsec, nrad = a.P.nrad, n0 = 2 * nrad;
  const size_t vs = 2 * sizeof(T);
  launch_k(a.pdl, sg_cols_fn<T>(a.sg_generic ? 0 : n0), dim3(a.sg.M), dim3(2 * sg_col_group(n0)), (n0 + 6 * fpadn(n0)) * vs, s, a);
  probe_mark(s, "k_sg_cols");
  launch_k(a.pdl, sg_rows_inv_fn<T>(a.sg_generic ? 0 : nsec), dim3(nrad), dim3(256), sg_rows_inv_smem<T>(nsec), s, a);
  probe_mark(s, "k_sg_rows_inv");
}

template <class T>
void launch_selfgravity(const KArgs<T> &a, cudaStream_t s) {
  launch_sg_rows_fwd(a, s);
  launch_sg_cols_inv(a, s);
}

// Set-up, FP64 in both modes: spectra of the constant kernels (compute_kernel
// src/SgMain.cu:49-81 is evaluated on the host; its transforms are done once
// here).  Azimuthal transforms of the 2 nrad rows of K^r, K^theta ...
__global__ void __launch_bounds__(256) k_sg_setup_rows(SgDev sg, int nsec, int n0) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char sg_raw[];
  double2 *b0 = (double2 *)sg_raw, *b1 = b0 + fpadn(nsec);
  const int i = blockIdx.x;
  for (int j = threadIdx.x; j < nsec; j += blockDim.x)
    b0[fpad(j)] = make_double2(sg.kr[(size_t)i * nsec + j], sg.kt[(size_t)i * nsec + j]);
  __syncthreads();
  double2 *Z = fft_run(b0, b1, nsec, sg.rad1, sg.nst1, sg.tw1_64, (int)threadIdx.x, (int)blockDim.x,
                       StoreFree<double2>());
  for (int m = threadIdx.x; m < sg.M; m += blockDim.x) {
    double2 xr, xt;
    unpack_pair(Z, m, nsec, xr, xt);
    sg.khat64_r[(size_t)m * n0 + i] = xr;
    sg.khat64_t[(size_t)m * n0 + i] = xt;
  }
}

// ... then the radial transform of each mode column, in place.
__global__ void __launch_bounds__(256) k_sg_setup_cols(SgDev sg, int n0) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char sg_raw[];
  double2 *b0 = (double2 *)sg_raw, *b1 = b0 + fpadn(n0);
  const int m = blockIdx.x;
  for (int f = 0; f < 2; f++) {
    double2 *kh = (f == 0 ? sg.khat64_r : sg.khat64_t) + (size_t)m * n0;
    for (int k = threadIdx.x; k < n0; k += blockDim.x) b0[fpad(k)] = kh[k];
    __syncthreads();
    double2 *X = fft_run(b0, b1, n0, sg.rad0, sg.nst0, sg.tw0_64, (int)threadIdx.x, (int)blockDim.x,
                         StoreFree<double2>());
    for (int k = threadIdx.x; k < n0; k += blockDim.x) kh[k] = X[fpad(k)];
    __syncthreads();
  }
}

// FP64 kernel spectra rounded to the per-step FFT type (FP32-bulk mode)
__global__ void k_sg_round_spectra(const double2 *__restrict__ in, float2 *__restrict__ out, size_t n) {
  pdl_enter();
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    out[k] = make_float2((float)in[k].x, (float)in[k].y);
}

template <class T>
void launch_sg_kernel_spectra(const KArgs<T> &a, cudaStream_t s) {
  const int nsec = a.P.nsec, n0 = 2 * a.P.nrad;
  k_sg_setup_rows<<<n0, 256, 2 * fpadn(nsec) * sizeof(double2), s>>>(a.sg, nsec, n0);
  k_sg_setup_cols<<<a.sg.M, 256, 2 * fpadn(n0) * sizeof(double2), s>>>(a.sg, n0);
  if (sizeof(T) == 4) {
    const size_t n = (size_t)a.sg.M * n0;
    k_sg_round_spectra<<<608, 256, 0, s>>>(a.sg.khat64_r, (float2 *)a.sg.khat_r, n);
    k_sg_round_spectra<<<608, 256, 0, s>>>(a.sg.khat64_t, (float2 *)a.sg.khat_t, n);
  }
}

template <class T>
cudaError_t prepare_sg_kernels(int nsec, int n0) {
  cudaError_t e;
  const int vs = 2 * sizeof(T);
  const int rows = (nsec + 2 * fpadn(nsec)) * vs, cols = (n0 + 6 * fpadn(n0)) * vs;
  const int rows64 = 2 * fpadn(nsec) * (int)sizeof(double2), cols64 = 2 * fpadn(n0) * (int)sizeof(double2);
  // the instances for these lengths and the run-time-plan ones
  for (int gen = 0; gen < 2; gen++) {
    const void *fr = (const void *)sg_rows_fwd_fn<T>(gen ? 0 : nsec), *fi = (const void *)sg_rows_inv_fn<T>(gen ? 0 : nsec),
               *fc = (const void *)sg_cols_fn<T>(gen ? 0 : n0);
    for (const void *f : {fr, fc, fi})
      if ((e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, FARGO_SMEM_CARVEOUT)) != cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(fr, cudaFuncAttributeMaxDynamicSharedMemorySize, rows)) != cudaSuccess) return e;
    if ((e = cudaFuncSetAttribute(fi, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sg_rows_inv_smem<T>(nsec))) != cudaSuccess)
      return e;
    if ((e = cudaFuncSetAttribute(fc, cudaFuncAttributeMaxDynamicSharedMemorySize, cols)) != cudaSuccess) return e;
  }
  if ((e = cudaFuncSetAttribute(k_sg_setup_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, rows64)) != cudaSuccess) return e;
  return cudaFuncSetAttribute(k_sg_setup_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, cols64);
}

#define INSTANTIATE_SG(T)                                                      \
  template void launch_selfgravity<T>(const KArgs<T> &, cudaStream_t);         \
  template void launch_sg_rows_fwd<T>(const KArgs<T> &, cudaStream_t);         \
  template void launch_sg_cols_inv<T>(const KArgs<T> &, cudaStream_t);         \
  template void launch_sg_kernel_spectra<T>(const KArgs<T> &, cudaStream_t);   \
  template cudaError_t prepare_sg_kernels<T>(int, int);
INSTANTIATE_SG(double)
INSTANTIATE_SG(float)
