// fargo_device.cuh -- device-side argument block and helpers for the step kernels.
#pragma once
#include <cuda.h>

#include <cuda_runtime.h>
#include <stdint.h>

#include "fargo_internal.h"

// Pointers of one disk as the kernels see them (passed by value).
template <class T>
struct DiskPtrs {
  // state
  T *dens, *vrad, *vtheta, *energy;
  // derived / scratch fields, (nrad+1)*nsec each unless noted
  T *cs;            // per-cell sound speed (energy equation) or nullptr
  T *pressure, *temperature, *potential;
  T *vradint, *vthetaint, *energyint;
  T *qplus, *divv, *taurr, *taurp, *taupp;
  T *densr, *energyr, *radmomp, *radmomm, *thetamomp, *thetamomm;
  T *sg_accr, *sg_acct;
  T *az_scratch;    // global fallback of the azimuthal kernel's ring buffers
  T *rdsum;         // FP64: 1/(rho + rho of the ring below), then 1/(rho + rho of the previous sector),
                    // formed by k_source for the substep's later kernels; nullptr for FP32
  // 1D tables
  const T *rt;      // RingTab rows in T
  const double *rt64;  // RingTab rows in FP64
  T *nu;            // viscosity profile (may be refreshed on the device)
  double *csmean;   // ring means of the sound speed (energy equation)
  const double *cosF, *sinF;  // force angle table (FP64)
  const T *cosFt, *sinFt;     // the same table in T
  const T *cosP, *sinP;       // potential angle table
  // per-ring partial results of the CFL/force kernel
  double *ring_force;
  double *lostbydisk;
  Ctl *ctl;
};

// Self-gravity FFT plan and buffers (fargo_sg.cu)
struct SgDev {
  // per-step buffers, complex of the field type (double2 or float2)
  void *spec_r, *spec_t;        // work spectra, [m][i], M x nrad
  void *spec2_r, *spec2_t;      // convolved spectra, [i][m], nrad x M
  void *khat_r, *khat_t;        // kernel spectra, [m][k], M x 2 nrad
  const void *tw1, *tw0;        // exp(-2 pi i t / N) for N = nsec and N = 2 nrad
  // set-up, FP64 (the same buffers as above in the FP64 mode)
  double2 *khat64_r, *khat64_t;
  const double2 *tw1_64, *tw0_64;
  const double *kr, *kt;        // real kernel tables, 2 nrad x nsec
  int rad1[16], nst1, rad0[16], nst0;
  int M;                        // nsec / 2 + 1
};

// TMA descriptors of the fields the radial transport reads (k_transport_radial_tma):
// 2D maps (sectors x rings 0..nrad) of the density, Vrad, Vtheta and energy.
struct RadMaps {
  CUtensorMap dens, vrad, vtheta, energy;
};

template <class T>
struct KArgs {
  DevParams P;
  DiskPtrs<T> d;
  double invdphi;      // 1.0/(2.0*M_PI/(double)nsec)
  double dtheta;       // 2.0*PI/(double)nsec
  double inv_nsec;     // 1.0/nsec
  double shear_k;      // 2.0*PI*CFLSECURITY/(double)nsec of the CFL shear limit
  // per-launch constants in both precisions (KC_*), read through KC()
  double k64[8];
  float k32[8];
  double lr01, lr12;   // log(Rmed[0]/Rmed[1]), log(Rmed[1]/Rmed[2]) for the Qplus extrapolation
  double nr_k1, nr_k2; // Rinf[1]^-1.5 - 1 and Rinf[nrad-2]^-1.5 - 1 of the non-reflecting boundary
  int mode;            // CFL/force kernel mode
  int az_smem;         // azimuthal kernel keeps its ring in shared memory
  int az_regs;         // register-blocked azimuthal kernel (nsec % 4 == 0)
  unsigned long long cond_handle;  // cudaGraphConditionalHandle of the DT while-loop
  int use_cond;                    // 1: k_end sets the while-loop condition
  int pdl;                         // launch with programmatic dependent launch
  int guard;                       // 1: return at once when the DT loop is done (a next substep's kernels)
  int sg_generic;                  // self-gravity FFTs with the run-time plan at every length
  const RadMaps *rad_maps;         // host copy of the radial transport's TMA maps (nullptr: plain loads)
  int rad_grid;                    // CTAs of the persistent TMA radial transport
  int cell_bx, cell_by;            // CTA shape (sectors x rings) of the per-cell kernels
  int az_chunks;                   // four-cell chunks per thread of the register azimuthal sweep
  int rad_col;                     // radial transport as a column march (k_transport_radial_col)
  SgDev sg;
};

// Sum accumulators of the reductions.  FP64 for T = double.  For T = float a
// float-float pair (Knuth's TwoSum per term, renormalised when two partial sums
// merge): about 44 significant bits from FP32 arithmetic, where this GPU issues
// FP64 at 1/64 of the FP32 rate.
template <class T>
struct SumAcc;

template <>
struct SumAcc<double> {
  double s;
  __device__ __forceinline__ void zero() { s = 0.0; }
  __device__ __forceinline__ void add(double x) { s += x; }
  __device__ __forceinline__ void merge(const SumAcc &o) { s += o.s; }
  __device__ __forceinline__ void merge_down(int o) { s += __shfl_down_sync(0xffffffffu, s, o); }
  __device__ __forceinline__ double value() const { return s; }
};

template <>
struct SumAcc<float> {
  float hi, lo;
  __device__ __forceinline__ void zero() { hi = lo = 0.0f; }
  __device__ __forceinline__ void add(float x) {
    const float t = hi + x, bb = t - hi;
    lo += (hi - (t - bb)) + (x - bb);
    hi = t;
  }
  __device__ __forceinline__ void merge(const SumAcc &o) {
    const float t = hi + o.hi, bb = t - hi;
    const float e = ((hi - (t - bb)) + (o.hi - bb)) + (lo + o.lo);
    hi = t + e;
    lo = e - (hi - t);
  }
  __device__ __forceinline__ void merge_down(int o) {
    SumAcc p;
    p.hi = __shfl_down_sync(0xffffffffu, hi, o);
    p.lo = __shfl_down_sync(0xffffffffu, lo, o);
    merge(p);
  }
  __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

template <class T>
__device__ __forceinline__ void warp_sum(SumAcc<T> &v) {
  for (int o = 16; o > 0; o >>= 1) v.merge_down(o);
}

// Block total of one SumAcc per thread; the result is valid in thread 0 only.
// sh: one SumAcc per warp.
template <class T>
__device__ __forceinline__ double block_total(SumAcc<T> v, SumAcc<T> *sh) {
  warp_sum(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < nw; k++) v.merge(sh[k]);
    return v.value();
  }
  return 0.0;
}

// The ring mean m as T arithmetic sees it: hi + lo with hi = (T)m (lo = 0 for FP64),
// so that x - m is formed as (x - hi) - lo.
template <class T>
struct RingMean {
  T hi, lo;
  __device__ __forceinline__ void set(double m) {
    hi = (T)m;
    lo = (T)(m - (double)hi);
  }
  __device__ __forceinline__ T sub_from(T x) const { return (x - hi) - lo; }
};
template <>
struct RingMean<double> {
  double hi, lo;
  __device__ __forceinline__ void set(double m) { hi = m; lo = 0.0; }
  __device__ __forceinline__ double sub_from(double x) const { return x - hi; }
};

enum { KC_GM1 = 0, KC_GGM1, KC_INVDPHI, KC_SGSELF, KC_DTHETA, KC_COUNT };

// control-block scalar in T: the FP32 copy for float kernels, the FP64 value otherwise
#define CTL_T(T, c, field, idx) (sizeof(T) == 4 ? (T)(c)->f32[idx] : (T)(c)->field)
// launch constant in T
#define KC(T, a, k) (sizeof(T) == 4 ? (T)(a).k32[k] : (T)(a).k64[k])

// Programmatic dependent launch: a step kernel launched with the attribute may
// be scheduled before the kernel ahead of it in the stream has finished; it
// first waits until that kernel has completed and its writes are visible.  The
// earlier kernel lets it launch only at its own exit (no explicit trigger: an
// early trigger parks waiting blocks on the SMs and slows the running kernel).
// A no-op for a kernel launched without the attribute.
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Four consecutive field values (16-byte aligned) in one or two vector accesses.
template <class T>
__device__ __forceinline__ void load4(const T *__restrict__ p, T *out);
template <>
__device__ __forceinline__ void load4<float>(const float *__restrict__ p, float *out) {
  const float4 v = *reinterpret_cast<const float4 *>(p);
  out[0] = v.x;
  out[1] = v.y;
  out[2] = v.z;
  out[3] = v.w;
}
template <>
__device__ __forceinline__ void load4<double>(const double *__restrict__ p, double *out) {
  const double2 v0 = *reinterpret_cast<const double2 *>(p), v1 = *reinterpret_cast<const double2 *>(p + 2);
  out[0] = v0.x;
  out[1] = v0.y;
  out[2] = v1.x;
  out[3] = v1.y;
}
template <class T>
__device__ __forceinline__ void store4(T *p, const T *v);
template <>
__device__ __forceinline__ void store4<float>(float *p, const float *v) {
  *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
template <>
__device__ __forceinline__ void store4<double>(double *p, const double *v) {
  reinterpret_cast<double2 *>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2 *>(p)[1] = make_double2(v[2], v[3]);
}

// FP64 division for the per-cell arithmetic of the FP64 mode, which is bound by
// GB300's narrow FP64 pipe.  Markstein's method (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000 processor", IBM J. Res. Dev.
// 34(1), 1990): the hardware reciprocal estimate (rcp.approx.ftz.f64), one
// Newton-Raphson step y' = y + y (1 - b y), the quotient q = a y', and one
// correction q' = q + (a - b q) y' with the residual formed exactly by a fused
// multiply-add.  Five FP64-pipe operations.  The corrected quotient is within about
// 2^-80 of a / b before its final rounding, so it is the correctly rounded quotient
// except where a / b lies that close to a rounding midpoint (then one ulp off).
// Outside |a|, |b| in [2^-500, 2^501) -- zero, subnormal, infinite or NaN operands,
// or a quotient that could leave the normal range -- it is IEEE a / b.
__device__ __forceinline__ double fdiv64(double a, double b) {
  const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu;
  const unsigned eb = ((unsigned)__double2hiint(b) >> 20) & 0x7ffu;
  if (ea - 523u > 1000u || eb - 523u > 1000u) return a / b;
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(b));
  y = fma(y, fma(-b, y, 1.0), y);
  const double q = a * y;
  return fma(fma(-b, q, a), y, q);
}

// Division in the bulk per-cell arithmetic: fdiv64 for double fields, IEEE
// division for float fields (the FP32-bulk arithmetic as before).
template <class T>
__device__ __forceinline__ T qdiv(T a, T b) { return a / b; }
template <>
__device__ __forceinline__ double qdiv<double>(double a, double b) { return fdiv64(a, b); }

// Division in the transport sweeps: the fast reciprocal-based divide for float
// fields (within 2 ulp; the FP32-bulk mode), fdiv64 for double fields.
__device__ __forceinline__ float bulk_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double bulk_div(double a, double b) { return fdiv64(a, b); }

// Division inside the van Leer slope limiters, 2 dq+ dq- / (dq+ + dq-)
// (StarRadKernel, StarThetaKernel): for double, fdiv64 without its correction
// step -- the reciprocal estimate, one Newton-Raphson step and the product, three
// FP64-pipe operations, relative error about 2^-40 (the estimate's 2^-20
// squared).  A limited slope enters a cell's new value only through the upwind
// interface correction (dxtheta -+ ksi) slope, which is bounded by the
// neighbouring differences of the quantity, so its 2^-40 error moves the updated
// fields by a few 1e-13 relative at most; a wrong sign or zero is impossible
// (the operands have one sign when the limiter divides).  Outside [2^-500,
// 2^501) it is IEEE a / b, as fdiv64.  For float: bulk_div.
__device__ __forceinline__ float lim_div(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double lim_div(double a, double b) {
  const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu;
  const unsigned eb = ((unsigned)__double2hiint(b) >> 20) & 0x7ffu;
  if (ea - 523u > 1000u || eb - 523u > 1000u) return a / b;
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(b));
  y = fma(y, fma(-b, y, 1.0), y);
  return a * y;
}

// Sign tests x > 0 and x < 0 of a non-NaN value.  For double, on the bit pattern
// with the integer pipe (a positive double is a positive 64-bit integer; a
// negative one other than -0 is an unsigned integer above 2^63), leaving the FP64
// pipe to the arithmetic; for float, the plain comparison.
template <class T>
__device__ __forceinline__ bool gt0(T x) { return x > (T)0; }
template <>
__device__ __forceinline__ bool gt0<double>(double x) { return __double_as_longlong(x) > 0LL; }
template <class T>
__device__ __forceinline__ bool lt0(T x) { return x < (T)0; }
template <>
__device__ __forceinline__ bool lt0<double>(double x) {
  return (unsigned long long)__double_as_longlong(x) > 0x8000000000000000ULL;
}
// x >= 0 of a non-NaN value (true for -0 as well), on the integer pipe for double
template <class T>
__device__ __forceinline__ bool ge0(T x) { return x >= (T)0; }
template <>
__device__ __forceinline__ bool ge0<double>(double x) { return !lt0(x); }
// The larger of two non-negative values: for double the integer order of the bit
// patterns, which is the order of non-negative doubles (no FP64-pipe compare).
template <class T>
__device__ __forceinline__ T max_nonneg(T x, T y) { return x > y ? x : y; }
template <>
__device__ __forceinline__ double max_nonneg<double>(double x, double y) {
  return __double_as_longlong(x) > __double_as_longlong(y) ? x : y;
}

// preferred shared-memory carveout (percent) of every step kernel
#define FARGO_SMEM_CARVEOUT 100

#define RT(a, row, i) ((a).d.rt[(i) * RT_COUNT + (row)])
#define RT64(a, row, i) ((a).d.rt64[(i) * RT_COUNT + (row)])

__device__ __forceinline__ double block_sum_d(double v, double *sh) {
  // sh: >= 32 doubles of shared memory; every thread gets the block sum
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < nw) ? sh[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[0] = v;
  }
  __syncthreads();
  double r = sh[0];
  __syncthreads();
  return r;
}

__device__ __forceinline__ double block_min_d(double v, double *sh) {
  for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (lane == 0) sh[w] = v;
  __syncthreads();
  if (w == 0) {
    v = (lane < nw) ? sh[lane] : 1e300;
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0) sh[0] = v;
  }
  __syncthreads();
  double r = sh[0];
  __syncthreads();
  return r;
}
