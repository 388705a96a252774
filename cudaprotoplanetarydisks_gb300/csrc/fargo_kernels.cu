// fargo_kernels.cu -- the hydro substep of FARGO-ADSG as sm_103a kernels.
//
// One substep (the body of the AlgoGas while loop, src/SourceEuler.cu:223-302)
// is this launch sequence on one stream, captured once in a CUDA graph:
//   k_cfl_forces        ConditionCFL + ComputeAccel(star, FeelDisk planets) + the
//                       planet part of FillForcesArrays; its last block decides
//                       dt and advances the planetary system (RK5, rotation)
//   [boundary kernels]  ApplyBoundaryCondition, when a boundary is open
//   [self-gravity]      fargo_sg.cu (azimuthal FFT, radial convolution, inverse)
//   k_source            ComputePressureField + Substep1Kernel + Update_sgvelocity
//   k_visc_tau          ViscousTermsKernel
//   k_visc_update       UpdateVelocitiesKernel + ApplySubKeplerianBoundaryKernel
//   k_artvisc           Substep2Kernel + kernel + ActualiseGasVrad/Vtheta
//   [k_energy]          ViscousTermsKernel on the new velocities + Substep3 (energy
//                       equation): the stresses stay in registers
//   k_transport_radial  LRMomenta + OneWindRad (all conserved quantities at once)
//                       (or k_transport_radial_tma / k_transport_radial_col)
//   k_transport_azimuthal  OneWindTheta: ring mean, FARGO split, two van Leer
//                       sweeps and the integer shift, one CTA per ring
//   k_velocities        ComputeVelocities (+ ComputeTemperatureField)
//   k_end               PhysicalTime, LostMass, while-loop condition
// Every kernel is templated on the field type T: double (FARGO_FP64, parity
// mode) or float (FARGO_FP32_BULK: FP64 kept for the CFL decision, the force
// sums, the planets, the ring means and the FARGO split).
#include <cuda_runtime.h>

#include "fargo_device.cuh"
#include "fargo_kernels.cuh"

#define PI FARGO_PI
#define CVNR FARGO_CVNR
#define CFLSECURITY FARGO_CFLSECURITY

namespace {

__device__ __forceinline__ int jm1(int j, int n) { return j == 0 ? n - 1 : j - 1; }
__device__ __forceinline__ int jp1(int j, int n) { return j == n - 1 ? 0 : j + 1; }

}  // namespace

// ---------------------------------------------------------------------------
// ConditionCFL (src/SourceEuler.cu:520-546, kernels src/Kernels.cu:1267-1359),
// ComputeAccel / ComputeForce (src/SideEuler.cu:242-255, src/Force.cu:372-405,
// ComputeForceKernel src/Kernels.cu:693-729) and the planet part of
// FillForcesArraysKernel (src/Kernels.cu:1226-1253).  One CTA of 256 threads per
// ring, one pass over the ring's cells for the CFL terms, the forces on the first
// two bodies and the potential; per-warp partial results meet in shared memory
// behind one barrier.  The last CTA to finish decides dt and totals the forces.
// mode 0: full substep start.  mode 1: CFL only (sloppy CFL at the DT start, or
// the ConditionCFL entry point).  mode 2: forces, dt = sloppy_dt.  mode 3: forces
// and potential only.
// FP64 divide and square root for the single-thread decisions at the end of a
// kernel: not inlined, so that the several calls share one copy of the code (run
// once per launch by the one CTA that finishes last, it is fetched cold, and
// instruction fetch, not arithmetic, sets its cost).  Same IEEE results.
__device__ __noinline__ double div_once(double a, double b) { return a / b; }
__device__ __noinline__ double sqrt_once(double x) { return sqrt(x); }

// Total over the rings of component v of the per-ring force partials (SumAcc<T>
// stored in 8 bytes), summed by one warp in a fixed order; valid in lane 0.
template <class T>
__device__ __forceinline__ double ring_total(const double *ring_force, int nrad, int nv, int v, int lane) {
  static_assert(sizeof(SumAcc<T>) == 8, "8-byte ring partials");
  SumAcc<T> s;
  s.zero();
#pragma unroll 8
  for (int k = lane; k < nrad; k += 32) {
    const double d = __ldcg(ring_force + (size_t)k * nv + v);
    SumAcc<T> x;
    memcpy(&x, &d, 8);
    s.merge(x);
  }
  warp_sum(s);
  return s.value();
}

// Inputs of one cell of the CFL/force pass.
template <class T>
struct CflCell {
  T vt, vtn, vr0, vr1, cs, dn, cf, sf, cp, sp;
};

// Per-ring values of the CFL/force pass.
template <class T>
struct CflRing {
  T rm, surf, invdrad, invdxt, invmind, cs;
  RingMean<T> vm;
};

template <class T>
__device__ __forceinline__ void cfl_cell_load(const KArgs<T> &a, int i, int j, bool cfl_ring, bool do_forces,
                                              CflCell<T> &q) {
  const int nsec = a.P.nsec;
  const size_t o = (size_t)i * nsec + j;
  q.vt = a.d.vtheta[o];
  q.vtn = q.vr0 = q.vr1 = q.cs = q.dn = q.cf = q.sf = q.cp = q.sp = (T)0;
  if (cfl_ring) {
    q.vtn = a.d.vtheta[(size_t)i * nsec + jp1(j, nsec)];
    q.vr0 = a.d.vrad[o];
    q.vr1 = a.d.vrad[o + nsec];
    if (a.d.cs) q.cs = a.d.cs[o];
  }
  if (do_forces) {
    q.dn = a.d.dens[o];
    q.cf = a.d.cosFt[j];
    q.sf = a.d.sinFt[j];
    if (a.P.nb > 0) {
      q.cp = a.d.cosP[j];
      q.sp = a.d.sinP[j];
    }
  }
}

// ConditionCFLKernel2D1 + 2D2 for one cell: the sum S of the squared inverse time
// steps.  min_j C/sqrt(S_j) = C/sqrt(max_j S_j) exactly (sqrt and division round
// monotonically), so only S_j is formed per cell, with per-ring reciprocals.
template <class T>
__device__ __forceinline__ T cfl_cell_S(const KArgs<T> &a, const CflCell<T> &q, const CflRing<T> &r) {
  const T vres = a.P.fast_transport ? r.vm.sub_from(q.vt) : q.vt;
  const T cs = a.d.cs ? q.cs : r.cs;
  const T invdt1 = cs * r.invmind;
  const T invdt2 = fabs(q.vr0) * r.invdrad;
  const T invdt3 = fabs(vres) * r.invdxt;
  T dvr = q.vr1 - q.vr0;
  T dvt = q.vtn - q.vt;
  // sign tests and the maximum on the integer pipe for FP64 (the same decisions)
  if (ge0(dvr)) dvr = (T)1e-10;
  else dvr = -dvr;
  if (ge0(dvt)) dvt = (T)1e-10;
  else dvt = -dvt;
  const T a4 = dvr * r.invdrad, b4 = dvt * r.invdxt;
  T invdt4 = max_nonneg(b4, a4);
  invdt4 *= (T)(4.0 * CVNR * CVNR);
  return invdt1 * invdt1 + invdt2 * invdt2 + invdt3 * invdt3 + invdt4 * invdt4;
}

// ComputeForceKernel term of one cell on one body (k = 0; all Hill-cut levels
// coincide since a = rh = 0): 1/d^3 from rsqrt, compensated or FP64 ring sums.
template <class T>
__device__ __forceinline__ void cell_force(T xc, T yc, T cellmass, T x, T y, T rs2, SumAcc<T> &fx, SumAcc<T> &fy) {
  const T dx = xc - x, dy = yc - y;
  const T ir = rsqrt(dx * dx + dy * dy + rs2);
  const T InvDist3 = ir * ir * ir;
  fx.add(cellmass * dx * InvDist3);
  fy.add(cellmass * dy * InvDist3);
}

// FP64 step bodies run out of line.  Each step body below is a template that the
// single-disk kernel (k_*) and the fused-ensemble kernel (kb_*) both run.  Inlined
// into two kernels, the same FP64 source can come out with different multiply-add
// pairs contracted into fused multiply-adds (every FP64 divide branches to the
// IEEE divide outside its safe exponent range, and the optimiser arranges those
// blocks per kernel), which moves the last bits.  For T = double the kernels
// therefore call one out-of-line instance of each body, so that both run the same
// machine code and the fused ensemble is bitwise the disks run alone; the FP32
// bodies stay inlined (their kernels agree bitwise inlined, tested).  The
// single-disk kernels take their arguments as __grid_constant__ so that the
// out-of-line call reads them in place.
#define FARGO_F64_BODY(body)                                                                    \
  template <class... X>                                                                         \
  __device__ __noinline__ void body##_f64(const KArgs<double> &a, const uint3 bid, X... x) {    \
    body<double>(a, bid, x...);                                                                 \
  }
#define FARGO_RUN_BODY(T, body, a, bid, ...)                                                   \
  do {                                                                                          \
    if constexpr (sizeof(T) == 8)                                                               \
      body##_f64(a, bid, ##__VA_ARGS__);                                                        \
    else                                                                                        \
      body<T>(a, bid, ##__VA_ARGS__);                                                           \
  } while (0)
#define FARGO_BID make_uint3(blockIdx.x, blockIdx.y, gridDim.x *gridDim.y)

// V4 = 1 (nsec % 4 == 0, 260 <= nsec <= 1024): thread t holds the inputs of cells
// 4t..4t+3 in registers, each stream read with one 16-byte load, in one batch
// ahead of the ring mean (one memory latency, a few load instructions).  V4 = 0:
// any nsec, 256 threads, cells j = tid, tid + 256, ... streamed.  Every sum runs
// in a fixed order, so each instance is deterministic.
// Per ring the CTA also folds the arguments of the two time-step limits into the
// control block's maxima (64-bit integer atomicMax on the bit patterns of
// positive doubles: order-free, so deterministic): the largest S of its cells
// (rings >= 1; limit C/sqrt(S)) and |Omega_i - Omega_i+1| (rings < nrad - 1; limit
// 2 pi C / nsec / |...|), with Omega_i+1 from the mean of ring i+1 summed in the
// same order as ring i+1's own CTA sums it.  Both limits are correctly rounded,
// monotone non-increasing maps, so the smallest limit over the rings is the map
// of the largest argument: the last CTA takes one sqrt and two divides of the two
// words it reads, and no other CTA waits on an FP64 divide.
template <class T, int V4>
__device__ __forceinline__ void cfl_forces_body(const KArgs<T> &a, const uint3 bid) {
  
  if (a.guard && a.d.ctl->done) return;  // the next substep's, after the DT's last
  constexpr int NW = 8;                       // most warps of a CTA (96 to 256 threads)
  constexpr int NV = 2 * (FARGO_MAXPL + 1);   // force components, body-major
  constexpr int NC = V4 ? 4 : 1;
  const DevParams &P = a.P;
  const int i = bid.x, nsec = P.nsec, nrad = P.nrad, tid = threadIdx.x;
  const int lane = tid & 31, w = tid >> 5, nw = blockDim.x >> 5;
  Ctl *c = a.d.ctl;
  __shared__ SumAcc<T> s_part[NW][NV];
  __shared__ SumAcc<T> s_vpart[2][NW];
  __shared__ T s_mx[NW];
  __shared__ T s_body[FARGO_MAXPL + 1][3];
  __shared__ T s_pot[FARGO_MAXPL][5];
  __shared__ double s_om[2];
  __shared__ RingMean<T> s_vm;
  __shared__ int s_nbody, s_last;
  __shared__ double s_ctl[6];  // DT, dtemp, sloppy_dt, PhysicalTime, err, done (read before any write)
  const bool do_cfl = (a.mode == 0 || a.mode == 1);
  const bool do_forces = (a.mode != 1);
  const bool do_step = (a.mode == 0 || a.mode == 2);
  const bool cfl_ring = do_cfl && i > 0;
  const bool shear_ring = do_cfl && i < nrad - 1;
  // the control scalars the last block's decision reads, fetched up front by
  // every block so that the last one has them at hand
  if (tid >= 64 && tid < 70) {
    const int k = tid - 64;
    s_ctl[k] = k == 0 ? c->DT : k == 1 ? c->dtemp : k == 2 ? c->sloppy_dt : k == 3 ? c->PhysicalTime
             : k == 4 ? (double)c->err : (double)c->done;
  }
  // planet parameters of this substep, computed after the previous planet update
  // (fargo_planet_params): bodies feeling the disk and the planets' potential terms
  if (do_forces) {
    if (tid <= FARGO_MAXPL) {
      s_body[tid][0] = (T)c->bx[tid];
      s_body[tid][1] = (T)c->by[tid];
      s_body[tid][2] = (T)c->brs2[tid];
    }
    if (tid >= 32 && tid < 32 + P.nb) {
      const int k = tid - 32;
      s_pot[k][0] = (T)c->px[k];
      s_pot[k][1] = (T)c->py[k];
      s_pot[k][2] = (T)c->pm[k];
      s_pot[k][3] = (T)c->ps2[k];
      s_pot[k][4] = (T)c->pinvd3[k];
    }
    if (tid == 0) s_nbody = c->nbody;
  }
  // per-ring table values, loaded with the cells (no load after a barrier)
  CflRing<T> r;
  r.rm = RT(a, RT_RMED, i);
  r.surf = RT(a, RT_SURF, i);
  r.invdrad = r.invdxt = r.invmind = r.cs = (T)0;
  r.vm.hi = r.vm.lo = (T)0;
  if (cfl_ring) {
    r.invdrad = RT(a, RT_INVDRAD, i);
    r.invdxt = RT(a, RT_INVDXTHETA_CFL, i);
    r.invmind = RT(a, RT_INVMIND, i);
    r.cs = a.d.cs ? (T)0 : RT(a, RT_CS, i);
  }
  const double inv_rm = (do_cfl && (tid == 0 || tid == 32)) ? RT64(a, RT_INVRMED, i + (tid >> 5)) : 0.0;
  const T *vth = a.d.vtheta + (size_t)i * nsec;
  const T *vth1 = vth + nsec;
  CflCell<T> q[NC];
  T vn[NC];
  const int j0 = 4 * tid;
  const bool own = V4 && j0 < nsec;
  if (own) {
    const size_t o = (size_t)i * nsec + j0;
    T x[4];
    load4(vth + j0, x);
#pragma unroll
    for (int c = 0; c < 4; c++) {
      q[c].vt = x[c];
      q[c].vtn = q[c].vr0 = q[c].vr1 = q[c].cs = q[c].dn = q[c].cf = q[c].sf = q[c].cp = q[c].sp = (T)0;
      vn[c] = (T)0;
    }
    if (cfl_ring) {
      load4(a.d.vrad + o, x);
#pragma unroll
      for (int c = 0; c < 4; c++) q[c].vr0 = x[c];
      load4(a.d.vrad + o + nsec, x);
#pragma unroll
      for (int c = 0; c < 4; c++) q[c].vr1 = x[c];
      if (a.d.cs) {
        load4(a.d.cs + o, x);
#pragma unroll
        for (int c = 0; c < 4; c++) q[c].cs = x[c];
      }
#pragma unroll
      for (int c = 0; c < 3; c++) q[c].vtn = q[c + 1].vt;
      q[3].vtn = vth[jp1(j0 + 3, nsec)];
    }
    if (do_forces) {
      load4(a.d.dens + o, x);
#pragma unroll
      for (int c = 0; c < 4; c++) q[c].dn = x[c];
      load4(a.d.cosFt + j0, x);
#pragma unroll
      for (int c = 0; c < 4; c++) q[c].cf = x[c];
      load4(a.d.sinFt + j0, x);
#pragma unroll
      for (int c = 0; c < 4; c++) q[c].sf = x[c];
      if (P.nb > 0) {
        load4(a.d.cosP + j0, x);
#pragma unroll
        for (int c = 0; c < 4; c++) q[c].cp = x[c];
        load4(a.d.sinP + j0, x);
#pragma unroll
        for (int c = 0; c < 4; c++) q[c].sp = x[c];
      }
    }
    if (shear_ring) load4(vth1 + j0, vn);
  }
  if (do_cfl) {
    // ConditionCFLKernel1D: ring means of Vtheta (ring i, and ring i+1 for the shear)
    SumAcc<T> v, v1;
    v.zero();
    v1.zero();
    if (V4) {
      if (own) {
#pragma unroll
        for (int c = 0; c < NC; c++) {
          v.add(q[c].vt);
          v1.add(vn[c]);
        }
      }
    } else {
      for (int j = tid; j < nsec; j += 256) v.add(vth[j]);
      if (shear_ring)
        for (int j = tid; j < nsec; j += 256) v1.add(vth1[j]);
    }
    warp_sum(v);
    if (lane == 0) s_vpart[0][w] = v;
    if (shear_ring) {
      warp_sum(v1);
      if (lane == 0) s_vpart[1][w] = v1;
    }
  }
  __syncthreads();
  if (do_cfl && (tid == 0 || (tid == 32 && shear_ring))) {
    const int h = tid >> 5;
    SumAcc<T> v = s_vpart[h][0];
    for (int k = 1; k < nw; k++) v.merge(s_vpart[h][k]);
    const double vmoy = sizeof(T) == 8 ? v.value() / (double)nsec : v.value() * a.inv_nsec;
    if (h == 0) s_vm.set(vmoy);
    // ring angular velocity of the shear limit (ConditionCFLKernel2D2)
    s_om[h] = vmoy * inv_rm;
  }
  if (do_cfl) __syncthreads();
  const int nbody = do_forces ? s_nbody : 0;
  if (cfl_ring) r.vm = s_vm;
  T *pot = a.d.potential + (size_t)i * nsec;
  T mx = (T)0.0;
  // the planets' potential of the register-resident cells, stored after the
  // last-block ticket (no later kernel of this launch reads it, so the fence
  // before the ticket need not wait for it)
  T ph[NC];
  const int nchunk = do_forces ? (nbody + 1) >> 1 : 1;
  for (int ch = 0; ch < nchunk; ch++) {
    const bool first = (ch == 0);
    const int b0 = 2 * ch;
    const bool two = do_forces && b0 + 1 < nbody;
    T x0 = (T)0, y0 = (T)0, r0 = (T)0, x1 = (T)0, y1 = (T)0, r1 = (T)0;
    if (do_forces) {
      x0 = s_body[b0][0];
      y0 = s_body[b0][1];
      r0 = s_body[b0][2];
    }
    if (two) {
      x1 = s_body[b0 + 1][0];
      y1 = s_body[b0 + 1][1];
      r1 = s_body[b0 + 1][2];
    }
    SumAcc<T> fx0, fy0, fx1, fy1;
    fx0.zero();
    fy0.zero();
    fx1.zero();
    fy1.zero();
    auto cell = [&](int j, const CflCell<T> &e, T &phk) {
      if (first && cfl_ring) {
        const T S = cfl_cell_S(a, e, r);
        mx = max_nonneg(S, mx);
      }
      if (do_forces) {
        const T cellmass = r.surf * e.dn;
        const T xc = r.rm * e.cf, yc = r.rm * e.sf;
        cell_force(xc, yc, cellmass, x0, y0, r0, fx0, fy0);
        if (two) cell_force(xc, yc, cellmass, x1, y1, r1, fx1, fy1);
        if (first && P.nb > 0) {
          // planet part of the potential (positions at the start of the substep)
          const T x = r.rm * e.cp, y = r.rm * e.sp;
          T phi = (T)0.0;
          for (int k = 0; k < P.nb; k++) {
            const T xp = s_pot[k][0], yp = s_pot[k][1], mp = s_pot[k][2];
            const T distance = (x - xp) * (x - xp) + (y - yp) * (y - yp);
            // -mp / sqrt(d^2 + eps^2) as -mp times one reciprocal square root (within
            // 1 ulp in FP64, 2 in FP32) instead of a square root and a divide
            T pt = -mp * rsqrt(distance + s_pot[k][3]);
            if (P.indirect_term) pt += mp * s_pot[k][4] * (x * xp + y * yp);
            phi += pt;
          }
          if (V4) phk = phi;
          else pot[j] = phi;
        }
      }
    };
    if (V4) {
      if (own) {
#pragma unroll
        for (int c = 0; c < NC; c++) cell(j0 + c, q[c], ph[c]);
      }
    } else {
      for (int j = tid; j < nsec; j += 256) {
        CflCell<T> e;
        cfl_cell_load(a, i, j, cfl_ring, do_forces, e);
        cell(j, e, ph[0]);
      }
    }
    if (do_forces) {
      warp_sum(fx0);
      warp_sum(fy0);
      if (two) {
        warp_sum(fx1);
        warp_sum(fy1);
      }
      if (lane == 0) {
        s_part[w][2 * b0] = fx0;
        s_part[w][2 * b0 + 1] = fy0;
        if (two) {
          s_part[w][2 * b0 + 2] = fx1;
          s_part[w][2 * b0 + 3] = fy1;
        }
      }
    }
  }
  if (cfl_ring) {
    for (int o = 16; o > 0; o >>= 1) {
      const T m2 = __shfl_down_sync(0xffffffffu, mx, o);
      mx = (m2 > mx) ? m2 : mx;
    }
    if (lane == 0) s_mx[w] = mx;
  }
  __syncthreads();
  if (tid < 2 * nbody) {
    // ring partial sums stay SumAcc<T> (8 bytes either way) until the totals
    SumAcc<T> f = s_part[0][tid];
    for (int k = 1; k < nw; k++) f.merge(s_part[k][tid]);
    reinterpret_cast<SumAcc<T> *>(a.d.ring_force)[(size_t)i * NV + tid] = f;
  }
  if (cfl_ring && tid == 32) {
    T m = s_mx[0];
    for (int k = 1; k < nw; k++) m = (s_mx[k] > m) ? s_mx[k] : m;
    const double S = (double)m;
    if (S > 0.0) atomicMax(&c->ring_max[0], __double_as_longlong(S));
  }
  if (shear_ring && tid == 64) {
    // NaN differences are skipped (d > 0 is false), as fmin skips them
    const double d = fabs(s_om[0] - s_om[1]);
    if (d > 0.0) atomicMax(&c->ring_max[1], __double_as_longlong(d));
  }
  // last block: CFL decision, force totals
  __threadfence();
  __syncthreads();
  if (tid == 0) s_last = (atomicAdd(&c->ticket, 1u) == bid.z - 1);
  if (own && do_forces && P.nb > 0) store4(pot + j0, ph);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  __shared__ double s_acc[NV];
  __shared__ double s_dtc[2];
  if (do_forces && w < 2) {
    // the disk's force on the star, one warp per component (fixed order,
    // deterministic); the planets' totals are formed by k_planets
    const double tot = ring_total<T>(a.d.ring_force, nrad, NV, w, lane);  // valid in lane 0
    if (lane == 0) s_acc[w] = tot;
  }
  if (do_cfl && (tid == 64 || tid == 65)) {
    // smallest per-ring step (CFL over the rings i >= 1, shear over i < nrad - 1)
    // from the largest argument; the maxima reset for the next launch
    const int k = tid - 64;
    const long long m = __ldcg(&c->ring_max[k]);
    c->ring_max[k] = FARGO_RING_NO_LIMIT;
    const double x = __longlong_as_double(m);
    s_dtc[k] = (m == FARGO_RING_NO_LIMIT) ? 1e30 : k == 0 ? div_once(CFLSECURITY, sqrt_once(x)) : div_once(a.shear_k, x);
  }
  __syncthreads();
  if (tid == 0) {
    c->ticket = 0u;
    double dt;
    bool cfl_err = false;
    // a substep entered with the DT already done pads a loop body of several
    // substeps: it runs with dt = 0, which leaves the disk and the planets as they
    // are, and takes no CFL decision
    const bool pad = do_step && s_ctl[5] != 0.0;
    if (pad) {
      dt = 0.0;
    } else if (do_cfl) {
      const double DeltaT = (a.mode == 1) ? s_ctl[0] : s_ctl[0] - s_ctl[1];
      double newdt = fmin(s_dtc[0], s_dtc[1]);
      if (DeltaT < newdt) newdt = DeltaT;
      double q = div_once(DeltaT, newdt);
      int cfl;
      if (!(q > 0.0) || !(q < 1.0e8)) {
        c->err |= FARGO_DEVERR_CFL;
        cfl_err = true;
        cfl = 1;
        c->done = 1;
      } else {
        cfl = (int)ceil(q);
      }
      c->cfl = cfl;
      dt = div_once(DeltaT, (double)cfl);
      if (a.mode == 1) c->sloppy_dt = dt;
    } else {
      dt = s_ctl[2];
    }
    if (do_forces) {
      // DiskOnPrimaryAcceleration, ComputeIndirectTerm (src/Pframeforce.cu:86-94)
      c->ind_x = P.indirect_term ? -s_acc[0] : 0.0;
      c->ind_y = P.indirect_term ? -s_acc[1] : 0.0;
      c->f32[CTL_F_INDX] = (float)c->ind_x;
      c->f32[CTL_F_INDY] = (float)c->ind_y;
      c->accx[0] = s_acc[0];
      c->accy[0] = s_acc[1];
    }
    if (do_step) {
      if (s_ctl[4] != 0.0 || cfl_err) dt = 0.0;
      c->dt = dt;
      c->f32[CTL_F_DT] = (float)dt;
      c->f32[CTL_F_INVDT] = dt != 0.0 ? 1.0f / (float)dt : 0.0f;
      if (!pad) {
        c->dtemp = s_ctl[1] + dt;
        c->nsub_dt += 1;
        c->dt_sub = dt;
      }
      c->padding = pad ? 1 : 0;
      c->t_sub = s_ctl[3];
    }
  }
  // FViscosity profile when it changes in time (a moving cavity)
  if (do_forces && P.nu_dynamic) {
    const double t = c->PhysicalTime, t0 = c->PhysicalTimeInitial;
    for (int k = tid; k < nrad; k += blockDim.x) {
      const T nu = (T)fargo_fviscosity(P, RT64(a, RT_RMED, k), a.d.csmean[k], t, t0);
      a.d.nu[k] = nu;
      a.d.nu[nrad + 1 + k] = nu != (T)0.0 ? qdiv((T)0.5, nu) : (T)0.0;  // 0.5 / nu of the heating term
    }
  }
}
template <int V4>
__device__ __noinline__ void cfl_forces_body_f64(const KArgs<double> &a, const uint3 bid) {
  cfl_forces_body<double, V4>(a, bid);
}
template <class T, int V4>
__device__ __forceinline__ void cfl_forces_run(const KArgs<T> &a, const uint3 bid) {
  if constexpr (sizeof(T) == 8)
    cfl_forces_body_f64<V4>(a, bid);
  else
    cfl_forces_body<T, V4>(a, bid);
}
template <class T, int V4>
__global__ void __launch_bounds__(256, V4 ? 1 : 2) k_cfl_forces(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  cfl_forces_run<T, V4>(a, FARGO_BID);
}

// The CFL/force kernel for a ring of nsec cells: four contiguous cells per
// thread when nsec % 4 == 0 and 260 <= nsec <= 1024 (96 to 256 threads: every
// single-thread role has tid < 96), else the streamed 256-thread form
template <class T>
void launch_cfl_forces(const KArgs<T> &a, cudaStream_t s) {
  const int nsec = a.P.nsec;
  const dim3 g(a.P.nrad);
  if (nsec % 4 == 0 && nsec >= 260 && nsec <= 1024)
    launch_k(a.pdl, k_cfl_forces<T, 1>, g, dim3((nsec / 4 + 31) / 32 * 32), 0, s, a);
  else
    launch_k(a.pdl, k_cfl_forces<T, 0>, g, dim3(256), 0, s, a);
}

// The planetary part of a substep (AdvanceSystemFromDisk, AdvanceSystemRK5,
// the corotating frame, RotatePsys; src/SourceEuler.cu:236-261) on one thread,
// from the disk accelerations, indirect term, dt and start time that
// k_cfl_forces left in the control block.  It writes only planet state and the
// next substep's planet parameters, which no hydro kernel of the substep reads,
// so it may run beside them; in a corotating frame the hydro kernels need the
// new frame rate and it runs before them.
__device__ __forceinline__ void planets_body(const DevParams &P, Ctl *c, const double *__restrict__ ring_force,
                                             int fp32) {
  constexpr int NV = 2 * (FARGO_MAXPL + 1);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nrad = P.nrad;
  // the disk's force on each planet feeling it (bodies 1.. of k_cfl_forces)
  for (int v = 2 + w; v < 2 * c->nbody; v += 2) {
    const double s = fp32 ? ring_total<float>(ring_force, nrad, NV, v, lane)
                          : ring_total<double>(ring_force, nrad, NV, v, lane);
    if (lane == 0) {
      if (v & 1) c->accy[v >> 1] = s;
      else c->accx[v >> 1] = s;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) fargo_planets_substep(*c, P, c->dt, c->t_sub);
}
__global__ void __launch_bounds__(64) k_planets(DevParams P, Ctl *c, const double *__restrict__ ring_force, int fp32) {
  pdl_enter();
  planets_body(P, c, ring_force, fp32);
}

// ---------------------------------------------------------------------------
// ComputeSoundSpeed (energy equation) + Make1Dprofile(1) ring means; one CTA per ring.
template <class T>
__device__ __forceinline__ void soundspeed_body(const KArgs<T> &a, const uint3 bid) {
  
  __shared__ SumAcc<T> s_red[8];
  const int i = bid.x, nsec = a.P.nsec;
  const double g = a.P.adiabaticindex;
  SumAcc<T> s;
  s.zero();
  for (int j = threadIdx.x; j < nsec; j += blockDim.x) {
    size_t q = (size_t)i * nsec + j;
    T cs = sqrt(qdiv(KC(T, a, KC_GGM1) * a.d.energy[q], a.d.dens[q]));
    a.d.cs[q] = cs;
    s.add(cs);
  }
  const double tot = block_total(s, s_red);
  if (threadIdx.x == 0) {
    const double m = tot / (double)nsec;
    a.d.csmean[i] = m;
    // FViscosity reads this ring mean (alpha viscosity): refresh the profile here,
    // where the sound speed changes
    if (a.P.viscosity_alpha) {
      const DevParams &P = a.P;
      const Ctl *c = a.d.ctl;
      const T nu = (T)(P.lambdadoubling == 0.0
                           ? P.alphaviscosity * m * m * RT64(a, RT_R15, i) * RT64(a, RT_CAVFAC, i)
                           : fargo_fviscosity(P, RT64(a, RT_RMED, i), m, c->PhysicalTime, c->PhysicalTimeInitial));
      a.d.nu[i] = nu;
      a.d.nu[P.nrad + 1 + i] = nu != (T)0.0 ? qdiv((T)0.5, nu) : (T)0.0;  // 0.5 / nu of the heating term
    }
  }
}
FARGO_F64_BODY(soundspeed_body)
template <class T>
__global__ void __launch_bounds__(256) k_soundspeed(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  FARGO_RUN_BODY(T, soundspeed_body, a, FARGO_BID);
}

// CorrectVthetaKernel src/Kernels.cu:1256-1263 (corotating frame)
template <class T>
__device__ __forceinline__ void correct_vtheta_body(const KArgs<T> &a, const uint3 bid) {
  
  const int j = bid.x * blockDim.x + threadIdx.x, i = bid.y * blockDim.y + threadIdx.y;
  if (i >= a.P.nrad || j >= a.P.nsec) return;
  const size_t q = (size_t)i * a.P.nsec + j;
  a.d.vtheta[q] = a.d.vtheta[q] - CTL_T(T, a.d.ctl, domega, CTL_F_DOMEGA) * RT(a, RT_RMED, i);
}
FARGO_F64_BODY(correct_vtheta_body)
template <class T>
__global__ void k_correct_vtheta(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  FARGO_RUN_BODY(T, correct_vtheta_body, a, FARGO_BID);
}

// ---------------------------------------------------------------------------
// Boundary conditions (ApplyBoundaryCondition src/SideEuler.cu:31-41)

// OpenBoundaryKernel src/Kernels.cu:482-495
template <class T>
__global__ void k_bc_open(KArgs<T> a) {
  pdl_enter();
  const int j = blockIdx.x * blockDim.x + threadIdx.x, nsec = a.P.nsec;
  if (j >= nsec) return;
  T *D = a.d.dens, *E = a.d.energy, *V = a.d.vrad;
  D[j] = D[nsec + j];
  E[j] = E[nsec + j];
  if (V[2 * nsec + j] > (T)0.0 || (D[nsec + j] < RT(a, RT_SIGMAMED, 0))) V[nsec + j] = (T)0.0;
  else V[nsec + j] = V[2 * nsec + j];
}

// NonReflectingBoundary src/SideEuler.cu:45-76 with kernels src/Kernels.cu:498-607,
// as four launches so that its FP64 work spreads over many SMs (one CTA would
// run it on one SM's FP64 pipe):
//   k_bc_nr_means(0): the ring means of the sound speed (rings 0, 1, nrad-1, nrad-2)
//   k_bc_nr_cells:    the shift of rings 0 and nrad-1 (NonReflectingBoundaryKernel)
//                     and the Vrad update (NonReflectingBoundaryKernel2)
//   k_bc_nr_means(1): the ring means of density and energy on rings 0 and nrad-1
//   k_bc_nr_adjust:   ReduceMean + MinusMeanKernel
// NonReflectingBoundaryKernel2 runs nsec2pot threads without a j < nsec guard; its
// extra threads write Vrad ring 2 (from ring 3) and ring nrad (from ring nrad-1
// after its update), as a launch whose threads run in increasing j would: the
// thread of cell j does both, reading old values before it writes them.  The
// sound-speed ring nrad read there is zero.
template <class T>
__device__ __forceinline__ double nr_cs(const KArgs<T> &a, int i, int j) {
  const int nsec = a.P.nsec;
  return a.d.cs ? (double)a.d.cs[(size_t)i * nsec + j] : (i < a.P.nrad ? (double)RT(a, RT_CS, i) : 0.0);
}

// the two shifts (in sectors) of the boundary rings from the sound-speed means
template <class T>
__device__ __forceinline__ void nr_angles(const KArgs<T> &a, const double *m, int &ia, int &ia2) {
  const int nsec = a.P.nsec, nrad = a.P.nrad;
  double dangle = a.nr_k1 / (.5 * (m[0] + m[1]));
  dangle *= (RT64(a, RT_RMED, 1) - RT64(a, RT_RMED, 0));
  ia = (int)(dangle / 2.0 / PI * (double)nsec + .5);
  double dangle2 = a.nr_k2 / (.5 * (m[2] + m[3]));
  dangle2 *= (RT64(a, RT_RMED, nrad - 1) - RT64(a, RT_RMED, nrad - 2));
  ia2 = (int)(dangle2 / 2.0 / PI * (double)nsec + .5);
}

// CTA r of 4: the FP64 mean of ring r's quantity into bc_mean[4 which + r]
template <class T>
__global__ void __launch_bounds__(256) k_bc_nr_means(KArgs<T> a, int which) {
  pdl_enter();
  __shared__ double s_red[32];
  const int nsec = a.P.nsec, nrad = a.P.nrad, r = blockIdx.x;
  double s = 0.0;
  if (which == 0) {
    const int ring = r == 0 ? 0 : r == 1 ? 1 : r == 2 ? nrad - 1 : nrad - 2;
    for (int j = threadIdx.x; j < nsec; j += blockDim.x) s += nr_cs(a, ring, j);
  } else {
    const T *src = (r & 2 ? a.d.energy : a.d.dens) + (size_t)(r & 1 ? nrad - 1 : 0) * nsec;
    for (int j = threadIdx.x; j < nsec; j += blockDim.x) s += (double)src[j];
  }
  const double tot = block_sum_d(s, s_red);
  // order of bc_mean[4..7]: density ring 0, density ring nrad-1, energy ring 0, energy ring nrad-1
  if (threadIdx.x == 0) a.d.ctl->bc_mean[4 * which + r] = tot / nsec;
}

template <class T>
__global__ void __launch_bounds__(256) k_bc_nr_cells(KArgs<T> a) {
  pdl_enter();
  const int nsec = a.P.nsec, nrad = a.P.nrad;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nsec) return;
  T *D = a.d.dens, *E = a.d.energy, *V = a.d.vrad;
  double m[4];
#pragma unroll
  for (int r = 0; r < 4; r++) m[r] = a.d.ctl->bc_mean[r];
  int ia, ia2;
  nr_angles(a, m, ia, ia2);
  // NonReflectingBoundaryKernel: ring 0 from ring 1 (shifted), ring nrad-1 from
  // ring nrad-2; the reference wraps a shift once (|shift| < nsec in practice), a
  // full modulo keeps every index inside the ring for any shift
  const int t = ((j + ia) % nsec + nsec) % nsec;
  D[t] = D[nsec + j];
  E[t] = E[nsec + j];
  const long ii = nrad - 1;
  const long src = (ii - 1) * nsec + (((j - ia2) % nsec + nsec) % nsec);
  D[ii * nsec + j] = D[src];
  E[ii * nsec + j] = E[src];
  // NonReflectingBoundaryKernel2 (ring 1 and ring nrad-1 read only rings 1, 2,
  // nrad-2, which no thread writes before these reads)
  const double sm1 = RT64(a, RT_SIGMAMED, 1), sm2 = RT64(a, RT_SIGMAMED, nrad - 2);
  const T v2 = V[2 * nsec + j];
  double vm = -nr_cs(a, 1, j) * ((double)D[nsec + j] - sm1) / sm1;
  V[nsec + j] = (T)(2.0 * vm - (double)v2);
  vm = nr_cs(a, (int)ii, j) * ((double)D[(ii - 1) * nsec + j] - sm2) / sm2;
  const T vlast = (T)(2. * vm - (double)V[(ii - 1) * nsec + j]);
  V[ii * nsec + j] = vlast;
  // ... its threads nsec + j < nsec2pot: Vrad ring 2 (after ring 1 read it) and
  // ring nrad (from ring nrad-1 as just updated, density after the shift)
  if (j < a.P.nsec2pot - nsec) {
    vm = -nr_cs(a, 2, j) * ((double)D[2 * nsec + j] - sm1) / sm1;
    V[2 * nsec + j] = (T)(2.0 * vm - (double)V[3 * nsec + j]);
    vm = nr_cs(a, nrad, j) * ((double)D[ii * nsec + j] - sm2) / sm2;
    V[(size_t)nrad * nsec + j] = (T)(2. * vm - (double)vlast);
  }
}

template <class T>
__global__ void __launch_bounds__(256) k_bc_nr_adjust(KArgs<T> a) {
  pdl_enter();
  const int nsec = a.P.nsec, nrad = a.P.nrad;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nsec) return;
  const double *md = a.d.ctl->bc_mean + 4;
  T *D = a.d.dens, *E = a.d.energy;
  const double s0 = RT64(a, RT_SIGMAMED, 0), s1 = RT64(a, RT_SIGMAMED, nrad - 1);
  const double e0 = RT64(a, RT_ENERGYMED, 0), e1 = RT64(a, RT_ENERGYMED, nrad - 1);
  D[j] += (T)(s0 - md[0]);
  E[j] += (T)(e0 - md[2]);
  D[(size_t)(nrad - 1) * nsec + j] += (T)(s1 - md[1]);
  E[(size_t)(nrad - 1) * nsec + j] += (T)(e1 - md[3]);
}

// EvanescentBoundary src/SideEuler.cu:104-123; kernel src/Kernels.cu:967-1015.
// Its SG term reads GLOBAL_bufarray_d, which the reference never fills (zero).
template <class T>
__global__ void k_bc_evanescent(KArgs<T> a) {
  pdl_enter();
  const DevParams &P = a.P;
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  const int nrad = P.nrad, nsec = P.nsec;
  if (i >= nrad || j >= nsec) return;
  const double rm = RT64(a, RT_RMED, i), r0 = RT64(a, RT_RMED, 0), rl = RT64(a, RT_RMED, nrad - 1);
  const double DRMIN = r0 * 1.25, DRMAX = rl * 0.84;
  if (!((rm < DRMIN) || (rm > DRMAX))) return;
  const Ctl *c = a.d.ctl;
  const double step = c->dt, t = c->PhysicalTime, t0 = c->PhysicalTimeInitial;
  const double Tin = 2.0 * PI * pow(r0, 3. / 2), Tout = 2.0 * PI * pow(rl, 3. / 2);
  double damping, lambda = 0.0;
  if (rm < DRMIN) {
    damping = (rm - DRMIN) / (r0 - DRMIN);
    lambda = damping * damping * 10.0 * step / Tin;
  }
  if (rm > DRMAX) {
    damping = (rm - DRMAX) / (rl - DRMAX);
    lambda = damping * damping * 10.0 * step / Tout;
  }
  const double AR = fargo_aspect_ratio(P, rm, t, t0);
  double vtheta0 = sqrt(1.0 * 1.0 / rm *
                        (1.0 - (1.0 + P.sigmaslope - 2.0 * P.flaringindex) * pow(AR, 2.0) * pow(rm, 2.0 * P.flaringindex)));
  vtheta0 -= rm * c->OmegaFrame;
  const double vrad0 = -3.0 * (double)a.d.nu[i] / rm * (-P.sigmaslope + .5);
  const double dens0 = RT64(a, RT_SIGMAMED, i), energy0 = RT64(a, RT_ENERGYMED, i);
  const size_t q = (size_t)i * nsec + j;
  a.d.vrad[q] = (T)(((double)a.d.vrad[q] + lambda * vrad0) / (1.0 + lambda));
  a.d.vtheta[q] = (T)(((double)a.d.vtheta[q] + lambda * vtheta0) / (1.0 + lambda));
  a.d.dens[q] = (T)(((double)a.d.dens[q] + lambda * dens0) / (1.0 + lambda));
  if (P.adiabatic) a.d.energy[q] = (T)(((double)a.d.energy[q] + lambda * energy0) / (1.0 + lambda));
}

// ---------------------------------------------------------------------------
// ComputePressureField (src/Kernels.cu:187-200) + Substep1Kernel (src/Kernels.cu:13-53)
// + Update_sgvelocityKernel (src/Kernels.cu:915-932) applied to VradInt/VthetaInt.
// The potential is the planet part written by k_cfl_forces plus the star term
// (direct + indirect) evaluated here; with no planet there is no star term, as in
// the reference (it is added inside the planet loop, src/Kernels.cu:1246).
// One cell of the source step: the new VradInt (ring > 0; zero on ring 0, which
// the reference never writes), VthetaInt and the pressure.
template <class T>
struct SrcCell {
  T vr, vt, p;
};
template <class T>
__device__ __forceinline__ SrcCell<T> source_cell(const KArgs<T> &a, int i, int j) {
  const DevParams &P = a.P;
  const int nsec = P.nsec;
  const Ctl *c = a.d.ctl;
  const T dt = CTL_T(T, c, dt, CTL_F_DT), Om = CTL_T(T, c, OmegaFrame, CTL_F_OMEGA);
  const T ix = CTL_T(T, c, ind_x, CTL_F_INDX), iy = CTL_T(T, c, ind_y, CTL_F_INDY);
  const int jm = jm1(j, nsec), jp = jp1(j, nsec);
  const size_t q = (size_t)i * nsec + j, qm = (size_t)i * nsec + jm;
  const T *D = a.d.dens, *E = a.d.energy, *PHI = a.d.potential;
  auto press = [&](size_t k, int ring) -> T {
    if (P.adiabatic) return KC(T, a, KC_GM1) * E[k];
    const T cs = a.d.cs ? a.d.cs[k] : RT(a, RT_CS, ring);
    return D[k] * cs * cs;
  };
  auto phi = [&](size_t k, int ring, int jj) -> T {
    if (P.nb == 0) return (T)0.0;
    const T rm = RT(a, RT_RMED, ring);
    const T x = rm * a.d.cosP[jj], y = rm * a.d.sinP[jj];
    T pot = -RT(a, RT_INVRMED, ring);
    pot -= ix * x + iy * y;
    return PHI[k] + pot;
  };
  SrcCell<T> o;
  const T p0 = press(q, i), pm = press(qm, i);
  const T f0 = phi(q, i, j), fm = phi(qm, i, jm);
  o.vr = (T)0.0;
  if (i > 0) {
    const T p1 = press(q - nsec, i - 1);
    const T f1 = phi(q - nsec, i - 1, j);
    const T idr = RT(a, RT_INVDIFFRMED, i);
    T gradp;
    if constexpr (sizeof(T) == 8) {
      // 1 / (rho + rho below) once per cell and substep, kept for the viscous update
      // and the artificial viscosity (within an ulp of each quotient)
      const T r = qdiv((T)1.0, D[q] + D[q - nsec]);
      a.d.rdsum[q] = r;
      gradp = (p0 - p1) * (T)2.0 * r * idr;
    } else {
      gradp = qdiv((p0 - p1) * (T)2.0, D[q] + D[q - nsec]) * idr;
    }
    T gradphi = (f0 - f1) * idr;
    const T *V = a.d.vtheta;
    T vt2 = V[q] + V[(size_t)i * nsec + jp] + V[q - nsec] + V[(size_t)(i - 1) * nsec + jp];
    vt2 = vt2 / (T)4.0 + Om * RT(a, RT_RINF, i);
    vt2 = vt2 * vt2;
    T vradint = -gradp - gradphi;
    T vradint2 = vradint + vt2 * RT(a, RT_INVRINF, i);
    T vr = a.d.vrad[q] + dt * vradint2;
    if (P.self_gravity) {
      const T *A = a.d.sg_accr;
      vr += dt * ((RT(a, RT_RINF, i) - RT(a, RT_RMED, i - 1)) * A[q] + (RT(a, RT_RMED, i) - RT(a, RT_RINF, i)) * A[q - nsec]) *
            idr;
    }
    o.vr = vr;
  }
  const T idx = RT(a, RT_INVDXTHETA, i);
  T gradp;
  if constexpr (sizeof(T) == 8) {
    // 1 / (rho + rho of the previous sector), kept likewise
    const T r = qdiv((T)1.0, D[q] + D[qm]);
    a.d.rdsum[(size_t)(a.P.nrad + 1) * nsec + q] = r;
    gradp = (p0 - pm) * (T)2.0 * r * idx;
  } else {
    gradp = qdiv((p0 - pm) * (T)2.0, D[q] + D[qm]) * idx;
  }
  T gradphi = (f0 - fm) * idx;
  T vt = a.d.vtheta[q] - dt * (gradp + gradphi);
  vt += dt * RT(a, RT_SUPPTORQUE, i);
  if (P.self_gravity) {
    // (j-1)%nsec is -1 at j = 0: the flat index i*nsec-1 (previous ring's last
    // cell); before the array at i = 0, taken as zero.
    const T prev = (q > 0) ? a.d.sg_acct[q - 1] : (T)0.0;
    vt += (T)0.5 * dt * (a.d.sg_acct[q] + prev);
  }
  o.vt = vt;
  o.p = p0;
  return o;
}

// ApplySubKeplerianBoundary (src/SideEuler.cu:296-320) at edge ring i, with the
// current ring mean of the sound speed in the self-gravity form (Make1Dprofile(1))
template <class T>
__device__ __forceinline__ T subkeplerian_edge(const KArgs<T> &a, int i) {
  const DevParams &P = a.P;
  const Ctl *c = a.d.ctl;
  const double r = RT64(a, RT_RMED, i);
  const double cm = P.self_gravity ? a.d.csmean[i] : 0.0;
  const double v = P.lambdadoubling == 0.0 ? sqrt(RT64(a, RT_VKEP2, i) - (P.self_gravity ? r * cm : 0.0))
                                           : fargo_vkep(P, r, c->PhysicalTime, c->PhysicalTimeInitial, cm);
  return (T)(v - r * c->OmegaFrame);
}

template <class T>
__device__ __forceinline__ void source_body(const KArgs<T> &a, const uint3 bid) {
  
  const int j = bid.x * blockDim.x + threadIdx.x, i = bid.y * blockDim.y + threadIdx.y;
  if (i >= a.P.nrad || j >= a.P.nsec) return;
  const SrcCell<T> o = source_cell(a, i, j);
  const size_t q = (size_t)i * a.P.nsec + j;
  if (i > 0) a.d.vradint[q] = o.vr;
  a.d.vthetaint[q] = o.vt;
  a.d.pressure[q] = o.p;
}
FARGO_F64_BODY(source_body)
template <class T>
__global__ void __launch_bounds__(256) k_source(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  FARGO_RUN_BODY(T, source_body, a, FARGO_BID);
}

// ViscousTermsKernel src/Kernels.cu:733-771 on (vr, vt) with the density dens, for
// one cell: the velocity divergence and the stresses (tau_rphi only for i > 0)
template <class T>
struct ViscCell {
  T divv, trr, tpp, trp;
};
template <class T>
__device__ __forceinline__ ViscCell<T> visc_tau_cell(const KArgs<T> &a, int i, int j, const T *__restrict__ vr,
                                                     const T *__restrict__ vt) {
  const int nsec = a.P.nsec;
  const int jm = jm1(j, nsec), jp = jp1(j, nsec);
  const size_t q = (size_t)i * nsec + j, qp = (size_t)i * nsec + jp, qm = (size_t)i * nsec + jm;
  const T *D = a.d.dens;
  const T invdphi = KC(T, a, KC_INVDPHI), onethird = (T)(1.0 / 3.0);
  const T irm = RT(a, RT_INVRMED, i), idrs = RT(a, RT_INVDIFFRSUP, i);
  const T drr = (vr[q + nsec] - vr[q]) * idrs;
  const T dpp = (vt[qp] - vt[q]) * invdphi * irm + (T)0.5 * (vr[q + nsec] + vr[q]) * irm;
  T divv = (vr[q + nsec] * RT(a, RT_RSUP, i) - vr[q] * RT(a, RT_RINF, i)) * idrs * irm;
  divv += (vt[qp] - vt[q]) * invdphi * irm;
  const T nu = a.d.nu[i];
  ViscCell<T> c;
  c.divv = divv;
  c.trr = (T)2.0 * D[q] * nu * (drr - onethird * divv);
  c.tpp = (T)2.0 * D[q] * nu * (dpp - onethird * divv);
  c.trp = (T)0.0;
  if (i > 0) {
    const T drp = (T)0.5 * (RT(a, RT_RINF, i) * (vt[q] * irm - vt[q - nsec] * RT(a, RT_INVRMED, i - 1)) * RT(a, RT_INVDIFFRMED, i) +
                            (vr[q] - vr[qm]) * invdphi * RT(a, RT_INVRINF, i));
    c.trp = (T)(2.0 * 0.25) * (D[q] + D[q - nsec] + D[qm] + D[qm - nsec]) * nu * drp;
  }
  return c;
}
template <class T>
__device__ __forceinline__ void visc_tau_body(const KArgs<T> &a, const uint3 bid, const T *__restrict__ vr, const T *__restrict__ vt) {
  const int j = bid.x * blockDim.x + threadIdx.x, i = bid.y * blockDim.y + threadIdx.y;
  const int nrad = a.P.nrad, nsec = a.P.nsec;
  if (i >= nrad || j >= nsec) return;
  const ViscCell<T> c = visc_tau_cell(a, i, j, vr, vt);
  const size_t q = (size_t)i * nsec + j;
  a.d.divv[q] = c.divv;
  a.d.taurr[q] = c.trr;
  a.d.taupp[q] = c.tpp;
  if (i > 0) a.d.taurp[q] = c.trp;
}
FARGO_F64_BODY(visc_tau_body)
template <class T>
__global__ void __launch_bounds__(256) k_visc_tau(const __grid_constant__ KArgs<T> a, const T *__restrict__ vr,
                                                  const T *__restrict__ vt) {
  pdl_enter();
  FARGO_RUN_BODY(T, visc_tau_body, a, FARGO_BID, vr, vt);
}

// UpdateVelocitiesKernel src/Kernels.cu:118-150 + ApplySubKeplerianBoundaryKernel
// src/Kernels.cu:1416-1430 (skipped with the evanescent boundary, src/SourceEuler.cu:338).
template <class T>
__device__ __forceinline__ void visc_update_body(const KArgs<T> &a, const uint3 bid) {
  
  const int j = bid.x * blockDim.x + threadIdx.x, i = bid.y * blockDim.y + threadIdx.y;
  const int nrad = a.P.nrad, nsec = a.P.nsec;
  if (i >= nrad || j >= nsec) return;
  const Ctl *c = a.d.ctl;
  const T dt = CTL_T(T, c, dt, CTL_F_DT);
  const int jm = jm1(j, nsec), jp = jp1(j, nsec);
  const size_t q = (size_t)i * nsec + j, qm = (size_t)i * nsec + jm, qp = (size_t)i * nsec + jp;
  const T *D = a.d.dens, *TRR = a.d.taurr, *TRP = a.d.taurp, *TPP = a.d.taupp;
  const T invdphi = KC(T, a, KC_INVDPHI);
  // x / (0.5 (rho + rho')): FP64 as 2 x times the reciprocal k_source kept
  auto div_half_sum = [&](T x, T dsum, const T *rsum) -> T {
    if constexpr (sizeof(T) == 8) return x * ((T)2.0 * *rsum);
    else return qdiv(x, (T)0.5 * dsum);
  };
  const size_t qt = (size_t)(nrad + 1) * nsec + q;
  if (i > 0 && i < nrad - 1) {
    a.d.vthetaint[q] += div_half_sum(dt * RT(a, RT_INVRMED, i) *
                                         ((RT(a, RT_RSUP, i) * TRP[q + nsec] - RT(a, RT_RINF, i) * TRP[q]) *
                                              RT(a, RT_INVDIFFRSUP, i) +
                                          (TPP[q] - TPP[qm]) * invdphi + (T)0.5 * (TRP[q] + TRP[q + nsec])),
                                     D[q] + D[qm], a.d.rdsum + qt);
  }
  if (i > 0) {
    a.d.vradint[q] += div_half_sum(dt * RT(a, RT_INVRINF, i) *
                                       ((RT(a, RT_RMED, i) * TRR[q] - RT(a, RT_RMED, i - 1) * TRR[q - nsec]) *
                                            RT(a, RT_INVDIFFRMED, i) +
                                        (TRP[qp] - TRP[q]) * invdphi - (T)0.5 * (TPP[q] + TPP[q - nsec])),
                                   D[q] + D[q - nsec], a.d.rdsum + q);
  }
  // (not in a padded substep, dt = 0: the edge rings keep the velocities the last
  // transport gave them)
  if (!a.P.evanescent && (i == 0 || i == nrad - 1) && dt != (T)0.0) a.d.vthetaint[q] = subkeplerian_edge(a, i);
}
FARGO_F64_BODY(visc_update_body)
template <class T>
__global__ void __launch_bounds__(256) k_visc_update(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  FARGO_RUN_BODY(T, visc_update_body, a, FARGO_BID);
}

// Substep2Kernel (src/Kernels.cu:409-434) + kernel (src/Kernels.cu:438-479) +
// ActualiseGasVrad/Vtheta: the artificial-viscosity pressures are evaluated where
// they are needed and the new velocities are written to Vrad/Vtheta directly.
template <class T>
__device__ __forceinline__ void artvisc_body(const KArgs<T> &a, const uint3 bid) {
  
  const int j = bid.x * blockDim.x + threadIdx.x, i = bid.y * blockDim.y + threadIdx.y;
  const int nrad = a.P.nrad, nsec = a.P.nsec;
  if (i >= nrad || j >= nsec) return;
  const T dt = CTL_T(T, a.d.ctl, dt, CTL_F_DT);
  const int jm = jm1(j, nsec), jp = jp1(j, nsec);
  const size_t q = (size_t)i * nsec + j, qm = (size_t)i * nsec + jm, qp = (size_t)i * nsec + jp;
  const T *D = a.d.dens, *VR = a.d.vradint, *VT = a.d.vthetaint;
  const T c2 = (T)(CVNR * CVNR);
  auto qr = [&](size_t k) -> T {
    T dv = VR[k + nsec] - VR[k];
    return lt0(dv) ? c2 * D[k] * dv * dv : (T)0.0;
  };
  auto qt = [&](size_t k, size_t kp) -> T {
    T dv = VT[kp] - VT[k];
    return lt0(dv) ? c2 * D[k] * dv * dv : (T)0.0;
  };
  const T qr0 = qr(q), qt0 = qt(q, qp);
  T vrnew = (T)0.0;
  if (i > 0) {
    const T qr1 = qr(q - nsec);
    const T densint = qr0 - qr1;
    // 2 dt / (rho + rho below): FP64 with the reciprocal k_source kept
    const T f = sizeof(T) == 8 ? dt * (T)2.0 * a.d.rdsum[q] : qdiv(dt * (T)2.0, D[q] + D[q - nsec]);
    vrnew = VR[q] - f * densint * RT(a, RT_INVDIFFRMED, i);
  }
  const T qtm = qt(qm, q);
  const T tempint = qt0 - qtm;
  const T idx = RT(a, RT_INVDXTHETA, i);
  const T f2 = sizeof(T) == 8 ? dt * (T)2.0 * a.d.rdsum[(size_t)(nrad + 1) * nsec + q] : qdiv(dt * (T)2.0, D[q] + D[qm]);
  const T vtnew = VT[q] - f2 * tempint * idx;
  if (a.P.adiabatic) {
    a.d.energyint[q] = a.d.energy[q] - dt * qr0 * (VR[q + nsec] - VR[q]) * RT(a, RT_INVDIFFRSUP, i) -
                       dt * qt0 * (VT[qp] - VT[q]) * idx;
  }
  a.d.vrad[q] = vrnew;
  a.d.vtheta[q] = vtnew;
  if (i == nrad - 1) {  // ghost ring of VradNew/VthetaNew is never written (zero)
    a.d.vrad[q + nsec] = (T)0.0;
    a.d.vtheta[q + nsec] = (T)0.0;
  }
}
FARGO_F64_BODY(artvisc_body)
template <class T>
__global__ void __launch_bounds__(256) k_artvisc(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  FARGO_RUN_BODY(T, artvisc_body, a, FARGO_BID);
}

// ViscousTermsKernel (src/Kernels.cu:733-771) on the new velocities + Substep3Kernel +
// Substep3Kernel2 (src/Kernels.cu:56-115) + ActualiseGasEnergy.
template <class T>
__device__ __forceinline__ void energy_body(const KArgs<T> &a, const uint3 bid) {
  
  const int j = bid.x * blockDim.x + threadIdx.x, i = bid.y * blockDim.y + threadIdx.y;
  const int nrad = a.P.nrad, nsec = a.P.nsec;
  if (i >= nrad || j >= nsec) return;
  const T dt = CTL_T(T, a.d.ctl, dt, CTL_F_DT);
  const T *D = a.d.dens;
  // ViscousTermsKernel on the new velocities (src/SourceEuler.cu:362-375), cell by
  // cell in registers: no stress field goes through memory
  const ViscCell<T> c0 = visc_tau_cell(a, i, j, a.d.vrad, a.d.vtheta);
  auto qplus = [&](int ii, const ViscCell<T> &c) -> T {
    const size_t k = (size_t)ii * nsec + j;
    const T nu = a.d.nu[ii];
    if (nu != (T)0.0) {
      // FP64: 0.5 / nu is the ring's, kept beside the profile where the profile is
      // formed (a divide fewer per cell on the FP64 pipe); FP32 divides in place
      // (cheaper than the extra load in this latency-bound kernel)
      const T hnu = sizeof(T) == 8 ? a.d.nu[nrad + 1 + ii] : qdiv((T)0.5, nu);
      T qp = qdiv(hnu, D[k]) * (c.trr * c.trr + c.trp * c.trp + c.tpp * c.tpp);
      qp += (T)(2.0 / 9.0) * nu * D[k] * c.divv * c.divv;
      return qp;
    }
    return (T)0.0;
  };
  T qp;
  if (i > 0) {
    qp = qplus(i, c0);
  } else if (a.d.nu[nrad - 1] != (T)0.0) {
    const T q1 = qplus(1, visc_tau_cell(a, 1, j, a.d.vrad, a.d.vtheta));
    const T q2 = qplus(2, visc_tau_cell(a, 2, j, a.d.vrad, a.d.vtheta));
    qp = q1 * exp(log(q1 / q2) * (T)a.lr01 / (T)a.lr12);
  } else {
    qp = (T)0.0;
  }
  const size_t q = (size_t)i * nsec + j;
  a.d.divv[q] = c0.divv;
  a.d.qplus[q] = qp;
  const T ei = a.d.energyint[q], dv = c0.divv;
  T enew;
  if (!a.P.cooling) {
    T num = dt * qp + ei;
    T den = (T)1.0 + KC(T, a, KC_GM1) * dt * dv;
    enew = qdiv(num, den);
  } else {
    // FP64: the two divisions by the ring's SigmaMed as products with its
    // reciprocal (within an ulp of the quotients).  FP32 divides: a per-ring
    // reciprocal rounded to FP32 is a bias of the same sign in every cell of the ring
    // and every substep, which the FP32 fields accumulate (measured: the density
    // error against FP64 after 2 DTs on the 1024 x 3072 disk grew 1.5e-5 -> 2.6e-5)
    const T em = RT(a, RT_ENERGYMED, i), ct = RT(a, RT_COOLTIME, i), qm = RT(a, RT_QPLUSMED, i);
    T num;
    if constexpr (sizeof(T) == 8) {
      const T ism = RT(a, RT_INVSIGMAMED, i);
      num = em * dt * D[q] * ism + ct * ei + dt * ct * (qp - qm * D[q] * ism);
    } else {
      const T sm = RT(a, RT_SIGMAMED, i);
      num = qdiv(em * dt * D[q], sm) + ct * ei + dt * ct * (qp - qdiv(qm * D[q], sm));
    }
    T den = dt + ct + KC(T, a, KC_GM1) * dt * ct * dv;
    enew = qdiv(num, den);
    if (dt == (T)0.0) enew = ei;  // a padded substep: (ct ei) / ct is not exactly ei
  }
  a.d.energy[q] = enew;
}
FARGO_F64_BODY(energy_body)
template <class T>
__global__ void __launch_bounds__(256) k_energy(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  FARGO_RUN_BODY(T, energy_body, a, FARGO_BID);
}

// ---------------------------------------------------------------------------
// Radial transport: LRMomentaKernel (src/Kernels.cu:774-787) + OneWindRad
// (src/TransportEuler.cu:60-156: StarRadKernel/2, DivisePolarGridKernel,
// VanLeerRadialKernel for every conserved quantity, density last), with no
// intermediate field in memory.  One CTA per 32 sectors x RAD_TR rings: the
// transported quantities of the tile and a halo of two rings go to shared
// memory, then the upwind values at the interfaces (each with the slope dq(k) of
// its upwind ring) and the cell updates are each formed once, one barrier between
// the phases.
#define RAD_NY 10  // thread rows: at most two rows per phase for every warp
#define RAD_NS 7   // streams: rmp, rmm, tmp, tmm, energy, density (as q/rho), raw density
#define RAD_SMEM(T) (sizeof(T) * 32 * (RAD_NS * (RAD_TR + 4) + 6 * RAD_TR + (RAD_TR + 1) + RAD_NS * (RAD_TR + 1)))

// The radial tile's shared arrays (32 sectors x RAD_TR rings and their halos).
template <class T>
struct RadTile {
  static constexpr int TW = 32, TR = RAD_TR, NS = RAD_NS;
  T (*sW)[TR + 4][TW];  // q/rho, rings i0-2 .. i0+TR+1
  T (*sQ)[TR][TW];      // raw quantities of the tile's rings
  T (*sV)[TW];          // Vrad at interfaces i0 .. i0+TR
  T (*sS)[TR + 1][TW];  // interface values at i0 .. i0+TR
  __device__ __forceinline__ explicit RadTile(unsigned char *smem) {
    sW = reinterpret_cast<T(*)[TR + 4][TW]>(smem);
    sQ = reinterpret_cast<T(*)[TR][TW]>(sW + NS);
    sV = reinterpret_cast<T(*)[TW]>(sQ + 6);
    sS = reinterpret_cast<T(*)[TR + 1][TW]>(sV + TR + 1);
  }
  // LRMomenta + DivisePolarGrid of one cell of row rr (ring i0-2+rr) into the tile
  __device__ __forceinline__ void put(int rr, int x, const T (&q)[6], T inv, T vr) const {
#pragma unroll
    for (int f = 0; f < 6; f++) sW[f][rr][x] = q[f] * inv;
    sW[6][rr][x] = q[5];
    if (rr >= 2 && rr < TR + 2) {
#pragma unroll
      for (int f = 0; f < 6; f++) sQ[f][rr - 2][x] = q[f];
    }
    if (rr >= 2 && rr <= TR + 2) sV[rr - 2][x] = vr;
  }
};

// ring-table rows of rings i0-1 .. i0+TR+1 (zero outside 0 .. nrad), staged with the
// tile so that no phase after a barrier loads from global memory
template <class T>
__device__ __forceinline__ void rad_stage_rt(const KArgs<T> &a, T (*sRT)[RAD_TR + 3], int i0, int x, int y) {
  const int nrad = a.P.nrad;
  if (y == 0 && x < RAD_TR + 3) {
    const int k = i0 - 1 + x;
    const bool ok = k >= 0 && k <= nrad;
    sRT[0][x] = ok ? RT(a, RT_INVDIFFRMED, k) : (T)0;
    sRT[1][x] = ok ? RT(a, RT_RMED, k) : (T)0;
    sRT[2][x] = ok ? RT(a, RT_RINF, k) : (T)0;
    sRT[3][x] = ok ? RT(a, RT_RSUP, k) : (T)0;
    sRT[4][x] = ok ? RT(a, RT_INVSURF, k) : (T)0;
  }
}

// StarRadKernel, StarRadKernel2 and VanLeerRadialKernel on a filled tile: the
// upwind interface values of every stream (each with its upwind ring's slope) and
// the cell updates, one barrier between the phases.
template <class T>
__device__ __forceinline__ void rad_tile_update(const KArgs<T> &a, const RadTile<T> &t, T (*sRT)[RAD_TR + 3],
                                                int i0, int j, int x, int y) {
  constexpr int TR = RAD_TR, NS = RAD_NS, ny = RAD_NY;
  const DevParams &P = a.P;
  const int nrad = P.nrad, nsec = P.nsec;
  const bool col = j < nsec;
  const T dt = CTL_T(T, a.d.ctl, dt, CTL_F_DT);
  const T dtheta = KC(T, a, KC_DTHETA);
  // StarRadKernel2 at the interfaces m = i0 .. i0+TR, with StarRadKernel's slope of
  // the upwind ring k (m-1 for v > 0, m otherwise; zero at the first and last ring)
  // formed where the interface needs it: one slope per interface and no pass of
  // its own
  for (int ss = y; ss < TR + 1; ss += ny) {
    const int m = i0 + ss;
    const bool in = m > 0 && m < nrad;
    const T v = t.sV[ss][x];
    // the upwind side and the coefficient of its slope, the same for every stream:
    // x(m-1) + lo/2 q'(m-1) for v > 0, x(m) - hi/2 q'(m) otherwise, formed as
    // lo (q'/2) and hi (q'/2) with half slopes (the same products: the factors 2
    // and 1/2 are exact)
    const bool up = gt0(v);
    T coef = (T)0.0;
    if (in) {
      const T lo = sRT[1][ss + 1] - sRT[1][ss] - v * dt;
      const T hi = sRT[1][ss + 2] - sRT[1][ss + 1] + v * dt;
      coef = up ? lo : -hi;
    }
    // the upwind ring's row in the slope numbering (ring i0-1+rd) and in sW (ring i0-2+rw)
    const int rd = up ? ss : ss + 1, rw = rd + 1;
    const int k = i0 - 1 + rd;
    const bool sl = in && k > 0 && k < nrad - 1;
    const T idm0 = sl ? sRT[0][rd] : (T)0.0, idm1 = sl ? sRT[0][rd + 1] : (T)0.0;
#pragma unroll
    for (int f = 0; f < NS; f++) {
      T d = (T)0.0;
      if (sl) {
        const T wm = t.sW[f][rw - 1][x], w0 = t.sW[f][rw][x], wp = t.sW[f][rw + 1][x];
        const T dqm = (w0 - wm) * idm0;
        const T dqp = (wp - w0) * idm1;
        d = gt0(dqp * dqm) ? lim_div(dqp * dqm, dqp + dqm) : (T)0.0;  // half the van Leer slope
      }
      const T sv = in ? t.sW[f][rw][x] + coef * d : (T)0.0;
      // the density's interface value enters only the mass flux through the
      // interface, dt dtheta Rinf(m) rho* v, the same for the cells on both sides
      // (Rsup of ring m-1 is Rinf of ring m): formed here once, in its slot
      t.sS[f][ss][x] = f < 6 ? sv : dt * dtheta * sRT[2][ss + 1] * sv * v;
    }
  }
  __syncthreads();
  if (!col) return;
  // VanLeerRadialKernel
  for (int r = y; r < TR; r += ny) {
    const int i = i0 + r;
    if (i >= nrad) break;
    const size_t q = (size_t)i * nsec + j;
    const T isurf = sRT[4][r + 1];
    // the mass fluxes through the cell's two interfaces, the same for every stream
    const T F0 = t.sS[6][r][x], F1 = t.sS[6][r + 1][x];
    T *out[6] = {a.d.radmomp, a.d.radmomm, a.d.thetamomp, a.d.thetamomm, a.d.energyr, a.d.densr};
#pragma unroll
    for (int f = 0; f < 6; f++) {
      if (f == 4 && !P.adiabatic) continue;
      const T varq = t.sS[f][r][x] * F0 - t.sS[f][r + 1][x] * F1;
      out[f][q] = t.sQ[f][r][x] + varq * isurf;
      if (f == 5 && i == 0 && P.open_inner) a.d.lostbydisk[j] = (double)varq;
    }
  }
}

// LRMomenta and DivisePolarGrid of one cell (ring k, sector j) from its inputs
template <class T>
__device__ __forceinline__ void rad_cell(const KArgs<T> &a, int k, T d, T v0, T v1, T vtp, T vt, T e, T (&q)[6],
                                         T &inv) {
  const T rm = RT(a, RT_RMED, k);
  const T Om = CTL_T(T, a.d.ctl, OmegaFrame, CTL_F_OMEGA);
  q[0] = d * v1;
  q[1] = d * v0;
  q[2] = d * (vtp + rm * Om) * rm;
  q[3] = d * (vt + rm * Om) * rm;
  q[4] = a.P.adiabatic ? e : (T)0.0;
  q[5] = d;
  inv = qdiv((T)1.0, d + (T)1e-20);
}

// out-of-line FP64 instances of the radial helpers, shared by the plain, the
// TMA-staged and the fused-ensemble radial kernels (see FARGO_F64_BODY)
template <class T>
struct RadCellOut {
  T q[6];
  T inv;
};
__device__ __noinline__ RadCellOut<double> rad_cell_f64(const KArgs<double> &a, int k, double d, double v0,
                                                        double v1, double vtp, double vt, double e) {
  RadCellOut<double> r;
  rad_cell<double>(a, k, d, v0, v1, vtp, vt, e, r.q, r.inv);
  return r;
}
template <class T>
__device__ __forceinline__ void rad_cell_run(const KArgs<T> &a, int k, T d, T v0, T v1, T vtp, T vt, T e,
                                             T (&q)[6], T &inv) {
  if constexpr (sizeof(T) == 8) {
    const RadCellOut<double> r = rad_cell_f64(a, k, d, v0, v1, vtp, vt, e);
#pragma unroll
    for (int f = 0; f < 6; f++) q[f] = r.q[f];
    inv = r.inv;
  } else {
    rad_cell<T>(a, k, d, v0, v1, vtp, vt, e, q, inv);
  }
}
__device__ __noinline__ void rad_tile_update_f64(const KArgs<double> &a, const RadTile<double> t,
                                                 double (*sRT)[RAD_TR + 3], int i0, int j, int x, int y) {
  rad_tile_update<double>(a, t, sRT, i0, j, x, y);
}
template <class T>
__device__ __forceinline__ void rad_tile_update_run(const KArgs<T> &a, const RadTile<T> &t, T (*sRT)[RAD_TR + 3],
                                                    int i0, int j, int x, int y) {
  if constexpr (sizeof(T) == 8)
    rad_tile_update_f64(a, t, sRT, i0, j, x, y);
  else
    rad_tile_update<T>(a, t, sRT, i0, j, x, y);
}

// Radial transport: LRMomentaKernel (src/Kernels.cu:774-787) + OneWindRad
// (src/TransportEuler.cu:60-156: StarRadKernel/2, DivisePolarGridKernel,
// VanLeerRadialKernel for every conserved quantity, density last), with no
// intermediate field in memory.  One CTA per 32 sectors x RAD_TR rings: the
// transported quantities of the tile and a halo of two rings go to shared
// memory, then the slopes dq(k) of the rings, the upwind values at the
// interfaces and the cell updates are each formed once, one barrier between
// the phases.
template <class T>
__device__ __forceinline__ void radial_body(const KArgs<T> &a, const uint3 bid) {
  
  constexpr int TR = RAD_TR, ny = RAD_NY;
  extern __shared__ __align__(128) unsigned char rad_smem[];
  const RadTile<T> t(rad_smem);
  const DevParams &P = a.P;
  const int nrad = P.nrad, nsec = P.nsec;
  const int x = threadIdx.x, y = threadIdx.y;
  const int j = bid.x * 32 + x, i0 = bid.y * TR;
  const bool col = j < nsec;
  const int jp = col ? jp1(j, nsec) : 0;
  __shared__ T sRT[5][TR + 3];  // INVDIFFRMED, RMED, RINF, RSUP, INVSURF
  rad_stage_rt(a, sRT, i0, x, y);
  // LRMomenta and DivisePolarGrid over the tile and its halo (zero outside the grid)
  for (int rr = y; rr < TR + 4; rr += ny) {
    const int k = i0 - 2 + rr;
    T q[6] = {(T)0, (T)0, (T)0, (T)0, (T)0, (T)0}, inv = (T)0.0, vr = (T)0.0;
    if (col && k >= 0 && k < nrad) {
      const size_t qk = (size_t)k * nsec + j;
      const T v0 = a.d.vrad[qk];
      rad_cell_run(a, k, a.d.dens[qk], v0, a.d.vrad[qk + nsec], a.d.vtheta[(size_t)k * nsec + jp], a.d.vtheta[qk],
               P.adiabatic ? a.d.energy[qk] : (T)0.0, q, inv);
      vr = v0;
    } else if (col && k == nrad) {
      vr = a.d.vrad[(size_t)k * nsec + j];
    }
    t.put(rr, x, q, inv, vr);
  }
  __syncthreads();
  rad_tile_update_run(a, t, sRT, i0, j, x, y);
}
template <class T>
__global__ void __launch_bounds__(32 * RAD_NY) k_transport_radial(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  radial_body<T>(a, make_uint3(blockIdx.x, blockIdx.y, gridDim.x * gridDim.y));
}

// ---------------------------------------------------------------------------
// The same radial transport as a column march.  The radial sweep couples a cell
// only to the cells of its own sector (and V_theta of the next sector), so one
// thread takes one sector and walks a chunk of RADC_RINGS rings upward, keeping
// the few rings its stencil needs in registers: the quantities over density of
// rings r-2, r-1, r, the slopes of rings r-2, r-1 and the upwind interface
// values at r-2, r-1.  No shared memory and no barrier: a warp's loads are 32
// consecutive sectors of one ring (coalesced), and the work per cell is the
// tile kernel's arithmetic in the same order (slopes, upwind values, updates).
// Each chunk re-reads the two rings on either side of it.  (Loading two rings
// ahead of their use measured slower at 1024 x 3072: 96 registers instead of 80,
// 98 us against 64 us a launch.)
template <class T>
struct RadColRing {
  T w[RAD_NS];  // q / (rho + 1e-20) for the six transported quantities, and rho itself
  T q[6];       // the raw quantities
  T v;          // Vrad at the ring's inner interface
};
// the loads of one cell (ring k)
template <class T>
struct RadColRaw {
  T d, v0, v1, vtp, vt, e;
};
template <class T>
__device__ __forceinline__ void radc_raw(const KArgs<T> &a, int k, int j, int jp, RadColRaw<T> &x) {
  const DevParams &P = a.P;
  const int nrad = P.nrad, nsec = P.nsec;
  x.d = x.v0 = x.v1 = x.vtp = x.vt = x.e = (T)0.0;
  if (k >= 0 && k < nrad) {
    const size_t qk = (size_t)k * nsec + j;
    x.d = a.d.dens[qk];
    x.v0 = a.d.vrad[qk];
    x.v1 = a.d.vrad[qk + nsec];
    x.vtp = a.d.vtheta[(size_t)k * nsec + jp];
    x.vt = a.d.vtheta[qk];
    if (P.adiabatic) x.e = a.d.energy[qk];
  } else if (k == nrad) {
    x.v0 = a.d.vrad[(size_t)k * nsec + j];
  }
}
// LRMomenta and DivisePolarGrid of ring k from its loads (zero outside the grid)
template <class T>
__device__ __forceinline__ void radc_form(const KArgs<T> &a, int k, const RadColRaw<T> &x, RadColRing<T> &c) {
  const int nrad = a.P.nrad;
#pragma unroll
  for (int f = 0; f < 6; f++) c.q[f] = (T)0;
  T inv = (T)0.0;
  c.v = (T)0.0;
  if (k >= 0 && k < nrad) {
    rad_cell_run(a, k, x.d, x.v0, x.v1, x.vtp, x.vt, a.P.adiabatic ? x.e : (T)0.0, c.q, inv);
    c.v = x.v0;
  } else if (k == nrad) {
    c.v = x.v0;
  }
#pragma unroll
  for (int f = 0; f < 6; f++) c.w[f] = c.q[f] * inv;
  c.w[6] = c.q[5];
}
// StarRadKernel at ring k from rings k-1, k, k+1 (zero at the first and last ring)
template <class T>
__device__ __forceinline__ void radc_slope(const KArgs<T> &a, int k, const RadColRing<T> &m, const RadColRing<T> &c,
                                           const RadColRing<T> &p, T (&d)[RAD_NS]) {
  const int nrad = a.P.nrad;
  const bool in = k > 0 && k < nrad - 1;
  const T idm0 = in ? RT(a, RT_INVDIFFRMED, k) : (T)0.0, idm1 = in ? RT(a, RT_INVDIFFRMED, k + 1) : (T)0.0;
#pragma unroll
  for (int f = 0; f < RAD_NS; f++) {
    T v = (T)0.0;
    if (in) {
      const T wm = m.w[f], w0 = c.w[f], wp = p.w[f];
      const T dqm = (w0 - wm) * idm0;
      const T dqp = (wp - w0) * idm1;
      v = gt0(dqp * dqm) ? lim_div(dqp * dqm, dqp + dqm) : (T)0.0;  // half the van Leer slope
    }
    d[f] = v;
  }
}
// StarRadKernel2 at interface m between rings m-1 (lo) and m (hi)
template <class T>
__device__ __forceinline__ void radc_iface(const KArgs<T> &a, int m, T dt, const RadColRing<T> &lo,
                                           const RadColRing<T> &hi, const T (&dlo)[RAD_NS], const T (&dhi)[RAD_NS],
                                           T (&sv)[RAD_NS]) {
  const int nrad = a.P.nrad;
  const bool in = m > 0 && m < nrad;
  const T v = hi.v;
  const bool up = gt0(v);
  T coef = (T)0.0;
  if (in) {
    const T r0 = RT(a, RT_RMED, m - 1), r1 = RT(a, RT_RMED, m), r2 = RT(a, RT_RMED, m + 1);
    const T l = r1 - r0 - v * dt;
    const T h = r2 - r1 + v * dt;
    coef = up ? l : -h;  // times the halved slope: l/2 q', -h/2 q'
  }
#pragma unroll
  for (int f = 0; f < RAD_NS; f++) sv[f] = in ? (up ? lo.w[f] + coef * dlo[f] : hi.w[f] + coef * dhi[f]) : (T)0.0;
}
template <class T>
__device__ __forceinline__ void radial_col_body(const KArgs<T> &a, const uint3 bid) {
  const DevParams &P = a.P;
  const int nrad = P.nrad, nsec = P.nsec;
  const int j = bid.x * RADC_THREADS + threadIdx.x;
  if (j >= nsec) return;
  const int jp = jp1(j, nsec);
  const int i0 = bid.y * RADC_RINGS, i1 = min(i0 + RADC_RINGS, nrad);
  const T dt = CTL_T(T, a.d.ctl, dt, CTL_F_DT);
  const T dtheta = KC(T, a, KC_DTHETA);
  T *const out[6] = {a.d.radmomp, a.d.radmomm, a.d.thetamomp, a.d.thetamomm, a.d.energyr, a.d.densr};
  // rings r-2, r-1, r; slopes of rings r-2, r-1; interface values at r-2, r-1
  RadColRing<T> c0, c1, c2;
  T d0[RAD_NS], d1[RAD_NS], s0[RAD_NS], s1[RAD_NS];
  {
    RadColRaw<T> x0, x1, x2, x3;  // the first four rings' loads, all in flight together
    radc_raw(a, i0 - 2, j, jp, x0);
    radc_raw(a, i0 - 1, j, jp, x1);
    radc_raw(a, i0, j, jp, x2);
    radc_raw(a, i0 + 1, j, jp, x3);
    radc_form(a, i0 - 2, x0, c0);
    radc_form(a, i0 - 1, x1, c1);
    radc_form(a, i0, x2, c2);
    radc_slope(a, i0 - 1, c0, c1, c2, d1);  // slope of ring i0-1
    // ring i0+1: slope of ring i0, interface value at i0
#pragma unroll
    for (int f = 0; f < RAD_NS; f++) d0[f] = d1[f];
    c0 = c1;
    c1 = c2;
    radc_form(a, i0 + 1, x3, c2);
    radc_slope(a, i0, c0, c1, c2, d1);
    radc_iface(a, i0, dt, c0, c1, d0, d1, s1);
  }
  // steady state: ring r, slope of ring r-1, interface at r-1, update of cell r-2
  T Fc = (T)0.0;  // the last cell's outer mass flux
  for (int r = i0 + 2; r <= i1 + 1; r++) {
#pragma unroll
    for (int f = 0; f < RAD_NS; f++) {
      d0[f] = d1[f];
      s0[f] = s1[f];
    }
    c0 = c1;
    c1 = c2;
    {
      RadColRaw<T> x;
      radc_raw(a, r, j, jp, x);
      radc_form(a, r, x, c2);
    }
    radc_slope(a, r - 1, c0, c1, c2, d1);
    radc_iface(a, r - 1, dt, c0, c1, d0, d1, s1);
    // VanLeerRadialKernel of cell i = r - 2 (ring c0)
    const int i = r - 2;
    const size_t q = (size_t)i * nsec + j;
    const T rsup = RT(a, RT_RSUP, i), isurf = RT(a, RT_INVSURF, i);
    // the cell's own interfaces: inner at i (s0), outer at i+1 (s1); Vrad at both.
    // The inner flux is the previous cell's outer one (Rinf of ring i is Rsup of
    // ring i-1), formed once
    const T v0 = c0.v, v1 = c1.v;
    const T F0 = r > i0 + 2 ? Fc : dt * dtheta * RT(a, RT_RINF, i) * s0[6] * v0;
    const T F1 = dt * dtheta * rsup * s1[6] * v1;
    Fc = F1;
#pragma unroll
    for (int f = 0; f < 6; f++) {
      if (f == 4 && !P.adiabatic) continue;
      const T varq = s0[f] * F0 - s1[f] * F1;
      out[f][q] = c0.q[f] + varq * isurf;
      if (f == 5 && i == 0 && P.open_inner) a.d.lostbydisk[j] = (double)varq;
    }
  }
}
FARGO_F64_BODY(radial_col_body)
template <class T>
__global__ void __launch_bounds__(RADC_THREADS) k_transport_radial_col(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  FARGO_RUN_BODY(T, radial_col_body, a, FARGO_BID);
}

// ---------------------------------------------------------------------------
// The same radial transport with its input tiles fetched by the Tensor Memory
// Accelerator.  A persistent CTA walks the 32-sector x RAD_TR-ring tiles of the
// grid (tile b, b + gridDim.x, ...).  Per tile, one thread issues four
// cp.async.bulk.tensor.2d copies (density, Vrad, Vtheta, energy: rings i0-2 ..
// i0+RAD_TR+2, sectors j0 .. j0+RAD_BW-1, zero-filled outside the field) into one
// of two shared-memory stages, completing on that stage's mbarrier, so the next
// tile streams in while this one is computed.  The cells are then formed from the
// staged tile exactly as k_transport_radial forms them from global memory (the
// azimuthal wrap of Vtheta at the last sector is the one plain load), and the
// phases after it are the same code: the results are bitwise equal.
#define RAD_FIELD_BYTES(T) (((size_t)RAD_BR * RAD_BW(T) * sizeof(T) + 127) / 128 * 128)
#define RAD_STAGE_BYTES(T) (4 * RAD_FIELD_BYTES(T))
#define RAD_TMA_SMEM(T) (((RAD_SMEM(T) + 127) / 128 * 128) + 2 * RAD_STAGE_BYTES(T) + 128)
// bounded waits: iterations of mbarrier.try_wait (each suspends the thread for a
// while in hardware) before the kernel gives up, flags the error and returns
#define TMA_WAIT_LIMIT (1u << 24)

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// waits for the phase `parity` of the mbarrier at `bar`; false after TMA_WAIT_LIMIT tries
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned parity) {
  for (unsigned n = 0; n < TMA_WAIT_LIMIT; n++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, unsigned bar, int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      :
      : "r"(smem_u32(dst)), "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

template <class T>
__global__ void __launch_bounds__(32 * RAD_NY) k_transport_radial_tma(const __grid_constant__ KArgs<T> a,
                                                                    const __grid_constant__ RadMaps maps) {
  pdl_enter();
  constexpr int TR = RAD_TR, ny = RAD_NY, BW = RAD_BW(T), BR = RAD_BR;
  extern __shared__ __align__(128) unsigned char rad_smem[];
  const RadTile<T> t(rad_smem);
  // the two stages start at the first 128-byte boundary after the tile's arrays
  // (RAD_TMA_SMEM holds 128 bytes of slack for it); each field box inside a stage
  // is a multiple of 128 bytes
  const unsigned smem_base = smem_u32(rad_smem);
  unsigned char *stage0 = rad_smem + ((((smem_base + (unsigned)RAD_SMEM(T)) + 127u) & ~127u) - smem_base);
  __shared__ __align__(8) unsigned long long bar[2];
  __shared__ T sRT[5][TR + 3];
  const DevParams &P = a.P;
  const int nrad = P.nrad, nsec = P.nsec;
  const int x = threadIdx.x, y = threadIdx.y, tid = y * 32 + x;
  const int ntx = (nsec + 31) / 32, nty = (nrad + TR - 1) / TR, ntiles = ntx * nty;
  const unsigned bytes = (unsigned)((P.adiabatic ? 4 : 3) * (size_t)BR * BW * sizeof(T));
  const CUtensorMap *fmaps[4] = {&maps.dens, &maps.vrad, &maps.vtheta, &maps.energy};
  auto field = [&](int s, int f) -> T(*)[BW] {
    return reinterpret_cast<T(*)[BW]>(stage0 + (size_t)s * RAD_STAGE_BYTES(T) + (size_t)f * RAD_FIELD_BYTES(T));
  };
  auto issue = [&](int tile, int s) {
    const unsigned b = smem_u32(&bar[s]);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    const int j0 = (tile % ntx) * 32, k0 = (tile / ntx) * TR - 2;
    for (int f = 0; f < 4; f++)
      if (f != 3 || P.adiabatic) tma_load_2d(field(s, f), fmaps[f], b, j0, k0);
  };
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if ((int)blockIdx.x < ntiles) issue(blockIdx.x, 0);
  }
  __syncthreads();
  int it = 0;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, it++) {
    const int s = it & 1;
    if (tid == 0 && tile + (int)gridDim.x < ntiles) issue(tile + gridDim.x, s ^ 1);
    const int j0 = (tile % ntx) * 32, i0 = (tile / ntx) * TR;
    const int j = j0 + x;
    const bool col = j < nsec;
    const int jp = col ? jp1(j, nsec) : 0;
    rad_stage_rt(a, sRT, i0, x, y);
    // every thread observes the stage's completion; the decision to give up is the
    // CTA's together (no thread leaves while others wait at a barrier)
    const bool ok = mbar_wait_bounded(smem_u32(&bar[s]), (unsigned)(it >> 1) & 1u);
    if (__syncthreads_or(!ok)) {
      // a copy did not complete: flag it, let the other stage's copy (if any) land
      // within the same bound, and stop
      if (tid == 0) {
        atomicOr(&a.d.ctl->err, FARGO_DEVERR_WAIT);
        if (tile + (int)gridDim.x < ntiles) mbar_wait_bounded(smem_u32(&bar[s ^ 1]), (unsigned)((it + 1) >> 1) & 1u);
      }
      return;
    }
    const T(*D)[BW] = field(s, 0);
    const T(*VR)[BW] = field(s, 1);
    const T(*VT)[BW] = field(s, 2);
    const T(*E)[BW] = field(s, 3);
    for (int rr = y; rr < TR + 4; rr += ny) {
      const int k = i0 - 2 + rr;
      T q[6] = {(T)0, (T)0, (T)0, (T)0, (T)0, (T)0}, inv = (T)0.0, vr = (T)0.0;
      if (col && k >= 0 && k < nrad) {
        const T v0 = VR[rr][x];
        // Vtheta at j+1: the next staged column, or sector 0 across the wrap
        const T vtp = (jp == j + 1) ? VT[rr][x + 1] : a.d.vtheta[(size_t)k * nsec];
        rad_cell_run(a, k, D[rr][x], v0, VR[rr + 1][x], vtp, VT[rr][x], P.adiabatic ? E[rr][x] : (T)0.0, q, inv);
        vr = v0;
      } else if (col && k == nrad) {
        vr = VR[rr][x];
      }
      t.put(rr, x, q, inv, vr);
    }
    __syncthreads();
    rad_tile_update_run(a, t, sRT, i0, j, x, y);
    __syncthreads();  // the tile and this stage are free for the next tiles
  }
}

// ---------------------------------------------------------------------------
// Azimuthal transport, one CTA per ring: OneWindTheta src/TransportEuler.cu:177-269
// with ComputeAverageThetaVelocities, ComputeResiduals, ComputeConstantResidual,
// QuantitiesAdvection (StarTheta/StarTheta2, DivisePolarGrid, VanLeerTheta) twice
// and AdvectSHIFT (src/Kernels.cu:1049-1190).  The ring lives in shared memory
// (or in global scratch when it does not fit); the FARGO shift is applied as an
// index rotation when the ring is stored.
#define AZ_NARR 12
template <class T>
__global__ void __launch_bounds__(512) k_transport_azimuthal(KArgs<T> a) {
  pdl_enter();
  extern __shared__ __align__(16) unsigned char az_smem[];
  __shared__ double s_red[32];
  __shared__ double s_vc;
  __shared__ int s_shift;
  const DevParams &P = a.P;
  const int i = blockIdx.x, nsec = P.nsec, tid = threadIdx.x, nt = blockDim.x;
  T *base = a.az_smem ? (T *)az_smem : a.d.az_scratch + (size_t)i * AZ_NARR * nsec;
  T *V = base, *Dn = base + nsec, *En = base + 2 * nsec, *M0 = base + 3 * nsec, *M1 = base + 4 * nsec,
    *M2 = base + 5 * nsec, *M3 = base + 6 * nsec, *W = base + 7 * nsec, *CF = base + 8 * nsec, *FL = base + 9 * nsec,
    *F = base + 10 * nsec, *ID = base + 11 * nsec;
  const Ctl *c = a.d.ctl;
  const double dt = c->dt;
  const size_t row = (size_t)i * nsec;
  // ComputeAverageThetaVelocitiesKernel (FP64 ring mean)
  double s = 0.0;
  for (int j = tid; j < nsec; j += nt) s += (double)a.d.vtheta[row + j];
  const double vmed = block_sum_d(s, s_red) / (double)nsec;
  if (tid == 0) {
    // ComputeConstantResidualKernel (FP64 split; Nshift is an integer decision)
    const double invdt = dt != 0.0 ? 1.0 / dt : 0.0;
    const double dpinvns = 2.0 * PI / (double)nsec;
    const double Ntilde = vmed * RT64(a, RT_INVRMED, i) * dt * (double)nsec / 2.0 / PI;
    const double Nround = floor(Ntilde + 0.5);
    s_shift = (int)(long)Nround;
    s_vc = (Ntilde - Nround) * RT64(a, RT_RMED, i) * invdt * dpinvns;
  }
  __syncthreads();
  const double vc = s_vc;
  const bool split = P.fast_transport;  // NoSplitAdvection == NO
  for (int j = tid; j < nsec; j += nt) {
    const double vt = (double)a.d.vtheta[row + j];
    V[j] = split ? (T)(vt - vmed) : (T)((vt - vmed) + vc);  // VthetaRes
    Dn[j] = a.d.densr[row + j];
    if (P.adiabatic) En[j] = a.d.energyr[row + j];
    M0[j] = a.d.radmomp[row + j];
    M1[j] = a.d.radmomm[row + j];
    M2[j] = a.d.thetamomp[row + j];
    M3[j] = a.d.thetamomm[row + j];
  }
  __syncthreads();
  const T dxtheta = RT(a, RT_DXTHETA, i), invdx = RT(a, RT_INVDXTHETA, i);
  const T dxrad = RT(a, RT_DRAD, i) * (T)dt, isurf = RT(a, RT_INVSURF, i);
  const T tdt = (T)dt;
  // StarThetaKernel: harmonic slope of q at cell j, times dxtheta (the 1/dxtheta
  // of the slope is carried by the upwind coefficient CF)
  auto slope_at = [&](const T *q, int j) -> T {
    const T dqm = q[j] - q[jm1(j, nsec)];
    const T dqp = q[jp1(j, nsec)] - q[j];
    return gt0(dqp * dqm) ? lim_div(dqp * dqm, dqp + dqm) : (T)0.0;
  };
  // QuantitiesAdvection with velocity vel[] (or the constant vconst).  Per
  // interface j (between cells j-1 and j) the upwind side, its slope coefficient
  // and the mass flux dxrad Dstar v are the same for every quantity: ksi = v dt is
  // kept in KS (the velocity's slot), the slope coefficient (dxtheta -+ ksi) /
  // dxtheta in CF and the flux factor in F, formed once per sweep; each quantity
  // then needs its W = Q / rho, its slopes, one upwind value and flux per
  // interface and its update (StarThetaKernel/2, DivisePolarGrid,
  // VanLeerThetaKernel, src/Kernels.cu:1049-1170).  Two barriers per quantity:
  // the update of one quantity and W of the next share a phase.  (The slope
  // times its coefficient is formed as coefficient x (dxtheta slope) instead of
  // (dxtheta -+ ksi) x slope: the same product to within an ulp of the
  // interface correction.)
  T *const KS = V;
  auto advect = [&](const T *vel, T vconst) {
    T *qs[6] = {M0, M1, M2, M3, En, Dn};
    int nf = 0, fs[6];
    for (int f = 0; f < 6; f++)
      if (f != 4 || P.adiabatic) fs[nf++] = f;
    // per interface j: the upwind cell c (j-1 or j) and its slope, formed where the
    // interface needs it (one slope per interface, as many as cells, and no pass
    // and barrier of their own)
    for (int j = tid; j < nsec; j += nt) {
      const T v = vel ? vel[j] : vconst;
      const T ksi = v * tdt;
      const bool up = gt0(ksi);
      const int c = up ? jm1(j, nsec) : j;
      const T cf = (up ? dxtheta - ksi : -(dxtheta + ksi)) * invdx;
      const T ds = Dn[c] + cf * slope_at(Dn, c);
      F[j] = dxrad * ds * v;
      KS[j] = ksi;  // vel[j] (== KS[j] in the first sweep) is read by this thread only
      CF[j] = cf;
      // DivisePolarGrid with the density's reciprocal, formed once per cell for every
      // quantity (one divide per cell instead of one per quantity, within an ulp)
      const T id = qdiv((T)1.0, Dn[j] + (T)1e-20);
      ID[j] = id;
      W[j] = qs[fs[0]][j] * id;
    }
    __syncthreads();
    for (int k = 0; k < nf; k++) {
      T *Q = qs[fs[k]];
      for (int j = tid; j < nsec; j += nt) {
        const int c = gt0(KS[j]) ? jm1(j, nsec) : j;
        FL[j] = (W[c] + CF[j] * slope_at(W, c)) * F[j];
      }
      __syncthreads();
      T *Qn = k + 1 < nf ? qs[fs[k + 1]] : nullptr;
      for (int j = tid; j < nsec; j += nt) {
        const T varq = FL[j] - FL[jp1(j, nsec)];
        Q[j] += varq * isurf;
        if (Qn) W[j] = Qn[j] * ID[j];
      }
      __syncthreads();
    }
  };
  advect(V, (T)0.0);
  if (split) advect(nullptr, (T)vc);
  // AdvectSHIFT: out[j] = q[(j - Nshift) mod nsec]
  int sh = s_shift % nsec;
  if (sh < 0) sh += nsec;
  for (int j = tid; j < nsec; j += nt) {
    int ji = j - sh;
    if (ji < 0) ji += nsec;
    a.d.dens[row + j] = Dn[ji];
    if (P.adiabatic) a.d.energy[row + j] = En[ji];
    a.d.radmomp[row + j] = M0[ji];
    a.d.radmomm[row + j] = M1[ji];
    a.d.thetamomp[row + j] = M2[ji];
    a.d.thetamomm[row + j] = M3[ji];
  }
}

// The same transport in registers, for nsec % 4 == 0: a thread owns chunks of
// four cells (chunk k = cells 4k..4k+3; thread t takes chunks t, t + blockDim,
// ..., one chunk each up to 768 FP32 / 512 FP64 threads, several on wider rings)
// and reads halos of two cells on either side from shared memory, so each sweep
// (slopes, upwind interface values and the update of all transported quantities,
// which depend only on themselves and on the old density) is one pass without
// barriers.  The first sweep writes a second copy of the
// ring, the second sweep (or the only one) stores to global memory at the
// shifted index.  Same per-cell arithmetic as k_transport_azimuthal.
namespace {
__device__ __forceinline__ int az_wrap(int j, int n) { return j < 0 ? j + n : (j >= n ? j - n : j); }
}  // namespace

#define AZ4_NARR 13
// threads of the register kernel: one per chunk of four cells, at most 768 (FP32)
// or 512 (FP64) (the register budget of one CTA per SM), whole warps
template <class T>
inline int az4_threads(int nsec) {
  const int most = sizeof(T) == 8 ? 512 : 768;
  const int n = nsec / 4 < most ? nsec / 4 : most;
  return (n + 31) / 32 * 32;
}
template <class T>
int az4_threads_host(int nsec) {
  return az4_threads<T>(nsec);
}
size_t rad_smem_bytes(int esize) { return esize == 8 ? RAD_SMEM(double) : RAD_SMEM(float); }
template <class T, bool MC>
__device__ __forceinline__ void azimuthal4_body(const KArgs<T> &a, const uint3 bid) {
  
  extern __shared__ __align__(16) unsigned char az_smem[];
  __shared__ SumAcc<T> s_part[32];
  __shared__ RingMean<T> s_vm;
  __shared__ T s_vct;
  __shared__ int s_shift;
  const DevParams &P = a.P;
  const int i = bid.x, nsec = P.nsec, tid = threadIdx.x;
  const int lane = tid & 31, w = tid >> 5, nw = (blockDim.x + 31) >> 5;
  const int nchunk = nsec >> 2;
  // body(j0) for the thread's chunks: one chunk in straight-line code when !MC
  auto each_chunk = [&](auto &&body) {
    if (MC) {
      for (int ch = tid; ch < nchunk; ch += (int)blockDim.x) body(4 * ch);
    } else if (tid < nchunk) {
      body(4 * tid);
    }
  };
  T *VT = (T *)az_smem;
  T *QA = VT + nsec;           // M0 M1 M2 M3 En Dn, nsec each
  T *QB = QA + 6 * nsec;       // the same after the first sweep
  const size_t row = (size_t)i * nsec;
  const T *src[6] = {a.d.radmomp, a.d.radmomm, a.d.thetamomp, a.d.thetamomm, a.d.energyr, a.d.densr};
  // the ring's table values and the control scalars, loaded with the ring (no
  // load after a barrier)
  const T tdt = CTL_T(T, a.d.ctl, dt, CTL_F_DT);
  const T dxtheta = RT(a, RT_DXTHETA, i), invdx = RT(a, RT_INVDXTHETA, i);
  const T dxrad = RT(a, RT_DRAD, i) * tdt, isurf = RT(a, RT_INVSURF, i);
  double azshift = 0.0, cdt = 0.0;
  T invdt = (T)0;
  if (tid == 0) {
    azshift = RT64(a, RT_AZSHIFT, i);
    cdt = a.d.ctl->dt;
    invdt = sizeof(T) == 4 ? (T)a.d.ctl->f32[CTL_F_INVDT] : (cdt != 0.0 ? (T)(1.0 / cdt) : (T)0);
  }
  // ring to shared memory; ComputeAverageThetaVelocitiesKernel
  SumAcc<T> vs;
  vs.zero();
  each_chunk([&](int j0) {
    T x[4];
    load4(a.d.vtheta + row + j0, x);
    store4(VT + j0, x);
#pragma unroll
    for (int c = 0; c < 4; c++) vs.add(x[c]);
#pragma unroll
    for (int f = 0; f < 6; f++) {
      if (f == 4 && !P.adiabatic) continue;
      load4(src[f] + row + j0, x);
      store4(QA + f * nsec + j0, x);
    }
  });
  warp_sum(vs);
  if (lane == 0) s_part[w] = vs;
  __syncthreads();
  if (tid == 0) {
    SumAcc<T> v = s_part[0];
    for (int k = 1; k < nw; k++) v.merge(s_part[k]);
    // ComputeAverageThetaVelocities + ComputeConstantResidual: the shift Nshift
    // is an FP64 integer decision; the constant residual velocity is a field
    // value, formed in T from the per-ring factor rm 2pi/nsec and 1/dt
    const double vmed = v.value() * a.inv_nsec;
    const double Ntilde = vmed * azshift * cdt;
    const double Nround = floor(Ntilde + 0.5);
    s_shift = (int)(long)Nround;
    s_vct = (T)(Ntilde - Nround) * dxtheta * invdt;
    s_vm.set(vmed);
  }
  __syncthreads();
  const T vct = s_vct;
  const bool split = P.fast_transport;  // NoSplitAdvection == NO
  int sh = s_shift % nsec;
  if (sh < 0) sh += nsec;
  const RingMean<T> vm = s_vm;
  // one sweep (QuantitiesAdvection) of the chunk at j0 from ring Q; out == nullptr:
  // store to global.
  // Per interface c (between cells j0-1+c and j0+c) the upwind side, the
  // coefficient of the upwind slope and the flux factor dxrad ds v are the same
  // for every quantity: formed once, then each quantity adds its slopes, its
  // upwind values and its update.
  auto sweep = [&](const T *Q, T *out, bool const_vel, int j0) {
    // VthetaRes at cells j0 .. j0+4
    // shared memory is read in whole chunks (16-byte accesses, no bank conflicts):
    // the thread's chunk and its neighbours' (the ring wraps chunk by chunk)
    const int jm = j0 == 0 ? nsec - 4 : j0 - 4, jp = j0 + 4 == nsec ? 0 : j0 + 4;
    T v[5];
    if (const_vel) {
#pragma unroll
      for (int c = 0; c < 5; c++) v[c] = vct;
    } else {
      T x[4];
      load4(VT + j0, x);
#pragma unroll
      for (int c = 0; c < 4; c++) v[c] = x[c];
      v[4] = VT[jp];
#pragma unroll
      for (int c = 0; c < 5; c++) {
        T vr = vm.sub_from(v[c]);
        if (!split) vr = vr + vct;
        v[c] = vr;
      }
    }
    // StarThetaKernel / StarThetaKernel2 on the density
    T d[8], id[8], dq[6], coef[5], F[5];
    bool upw[5];
    // cells j0-2 .. j0+5 of ring quantity f: two of the previous chunk, the
    // thread's chunk, two of the next
    // (FP64: element by element, which needs fewer live registers)
    auto halo8 = [&](const T *qf, T (&h)[8]) {
      if (sizeof(T) == 4) {
        T x[4];
        load4(qf + jm, x);
        h[0] = x[2];
        h[1] = x[3];
        load4(qf + j0, x);
#pragma unroll
        for (int c = 0; c < 4; c++) h[2 + c] = x[c];
        load4(qf + jp, x);
        h[6] = x[0];
        h[7] = x[1];
      } else {
#pragma unroll
        for (int c = 0; c < 8; c++) h[c] = qf[az_wrap(j0 - 2 + c, nsec)];
      }
    };
    halo8(Q + 5 * nsec, d);
#pragma unroll
    for (int c = 0; c < 8; c++) id[c] = bulk_div((T)1.0, d[c] + (T)1e-20);  // DivisePolarGrid: one reciprocal per cell
    // slopes times dxtheta; the upwind coefficient carries the 1/dxtheta
#pragma unroll
    for (int k = 0; k < 6; k++) {
      const T dqm = d[k + 1] - d[k], dqp = d[k + 2] - d[k + 1];
      dq[k] = gt0(dqp * dqm) ? lim_div(dqp * dqm, dqp + dqm) : (T)0.0;
    }
#pragma unroll
    for (int c = 0; c < 5; c++) {
      const T ksi = v[c] * tdt;
      upw[c] = gt0(ksi);
      // x + (dxtheta - ksi) q' upwind from the left, x - (dxtheta + ksi) q' from the right
      coef[c] = (upw[c] ? dxtheta - ksi : -(dxtheta + ksi)) * invdx;
      const T ds = (upw[c] ? d[c + 1] : d[c + 2]) + coef[c] * (upw[c] ? dq[c] : dq[c + 1]);
      F[c] = dxrad * ds * v[c];
    }
#pragma unroll
    for (int f = 0; f < 6; f++) {
      if (f == 4 && !P.adiabatic) continue;
      const T *q = Q + f * nsec;
      T *dst = f == 0 ? a.d.radmomp
             : f == 1 ? a.d.radmomm
             : f == 2 ? a.d.thetamomp
             : f == 3 ? a.d.thetamomm
             : f == 4 ? a.d.energy
                      : a.d.dens;
      T qv[8], wv[8], dw[6], sw[5];
      halo8(q, qv);
#pragma unroll
      for (int c = 0; c < 8; c++) {
        // DivisePolarGrid with the density's reciprocal, formed once per cell for
        // every quantity (FP64: one divide per cell instead of one per quantity,
        // within an ulp of q / rho)
        wv[c] = qv[c] * id[c];
      }
#pragma unroll
      for (int k = 0; k < 6; k++) {
        const T dqm = wv[k + 1] - wv[k], dqp = wv[k + 2] - wv[k + 1];
        dw[k] = gt0(dqp * dqm) ? lim_div(dqp * dqm, dqp + dqm) : (T)0.0;
      }
#pragma unroll
      for (int c = 0; c < 5; c++) sw[c] = (upw[c] ? wv[c + 1] : wv[c + 2]) + coef[c] * (upw[c] ? dw[c] : dw[c + 1]);
      T nq[4];
#pragma unroll
      for (int c = 0; c < 4; c++) {
        const T varq = sw[c] * F[c] - sw[c + 1] * F[c + 1];
        nq[c] = qv[2 + c] + varq * isurf;
      }
      if (out) {
        store4(out + f * nsec + j0, nq);
      } else {
#pragma unroll
        for (int c = 0; c < 4; c++) {
          // AdvectSHIFT: out[j] = q[(j - Nshift) mod nsec]
          int jo = j0 + c + sh;
          if (jo >= nsec) jo -= nsec;
          dst[row + jo] = nq[c];
        }
      }
    }
  };
  if (split) {
    each_chunk([&](int j0) { sweep(QA, QB, false, j0); });
    __syncthreads();
    each_chunk([&](int j0) { sweep(QB, nullptr, true, j0); });
  } else {
    each_chunk([&](int j0) { sweep(QA, nullptr, false, j0); });
  }
}
template <bool MC>
__device__ __noinline__ void azimuthal4_body_f64(const KArgs<double> &a, const uint3 bid) {
  azimuthal4_body<double, MC>(a, bid);
}
template <class T, bool MC>
__device__ __forceinline__ void azimuthal4_run(const KArgs<T> &a, const uint3 bid) {
  if constexpr (sizeof(T) == 8)
    azimuthal4_body_f64<MC>(a, bid);
  else
    azimuthal4_body<T, MC>(a, bid);
}
template <class T, bool MC>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 512 : 768) k_transport_azimuthal4(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  azimuthal4_run<T, MC>(a, FARGO_BID);
}

// ComputeVelocitiesKernel src/Kernels.cu:1193-1210 (+ ComputeTemperatureFieldKernel
// src/Kernels.cu:203-213 when no boundary runs in between).
template <class T>
__device__ __forceinline__ void velocities_body(const KArgs<T> &a, const uint3 bid, int with_temperature) {
  
  const int j = bid.x * blockDim.x + threadIdx.x, i = bid.y * blockDim.y + threadIdx.y;
  const int nrad = a.P.nrad, nsec = a.P.nsec;
  if (i >= nrad || j >= nsec) return;
  const T Om = CTL_T(T, a.d.ctl, OmegaFrame, CTL_F_OMEGA), dt = CTL_T(T, a.d.ctl, dt, CTL_F_DT);
  const int jm = jm1(j, nsec);
  const size_t q = (size_t)i * nsec + j, qm = (size_t)i * nsec + jm;
  const T *D = a.d.dens;
  const T vr = (i == 0) ? (T)0.0 : qdiv(a.d.radmomp[q - nsec] + a.d.radmomm[q], D[q] + D[q - nsec] + (T)1e-20);
  const T rm = RT(a, RT_RMED, i);
  // FP64: the division by Rmed as the product with its reciprocal (within an ulp);
  // FP32 divides (a per-ring FP32 reciprocal biases every substep the same way)
  const T w = qdiv(a.d.thetamomp[qm] + a.d.thetamomm[q], D[q] + D[qm] + (T)1e-15);
  const T vt = (sizeof(T) == 8 ? w * RT(a, RT_INVRMED, i) : qdiv(w, rm)) - rm * Om;
  // a substep with dt = 0 (a padded one) keeps the velocities: re-deriving them
  // from the momenta is not exact
  if (dt != (T)0.0) {
    a.d.vrad[q] = vr;
    a.d.vtheta[q] = vt;
  }
  if (with_temperature) {
    if (!a.P.adiabatic) a.d.temperature[q] = qdiv(a.d.pressure[q], D[q]);
    else a.d.temperature[q] = qdiv(KC(T, a, KC_GM1) * a.d.energy[q], D[q]);
  }
  if (!isfinite(D[q])) atomicOr(&a.d.ctl->err, FARGO_DEVERR_NAN);
}
FARGO_F64_BODY(velocities_body)
template <class T>
__global__ void __launch_bounds__(256) k_velocities(const __grid_constant__ KArgs<T> a, int with_temperature) {
  pdl_enter();
  FARGO_RUN_BODY(T, velocities_body, a, FARGO_BID, with_temperature);
}

// ComputeTemperatureFieldKernel src/Kernels.cu:203-213 (after a boundary condition)
template <class T>
__global__ void k_temperature(KArgs<T> a) {
  pdl_enter();
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= a.P.nrad || j >= a.P.nsec) return;
  const size_t q = (size_t)i * a.P.nsec + j;
  if (!a.P.adiabatic) a.d.temperature[q] = a.d.pressure[q] / a.d.dens[q];
  else a.d.temperature[q] = KC(T, a, KC_GM1) * a.d.energy[q] / a.d.dens[q];
}

// End of a substep: LostMass (src/TransportEuler.cu:77), PhysicalTime += dt
// (src/SourceEuler.cu:302) and the while-loop condition of AlgoGas (line 222).
template <class T>
__device__ __forceinline__ void end_body(const KArgs<T> &a, const uint3 bid) {
  
  __shared__ double s_red[32];
  Ctl *c = a.d.ctl;
  if (a.P.open_inner) {
    double s = 0.0;
    for (int j = threadIdx.x; j < a.P.nsec; j += blockDim.x) s += a.d.lostbydisk[j];
    s = block_sum_d(s, s_red);
    if (threadIdx.x == 0) c->LostMass += s;
  }
  if (threadIdx.x == 0 && c->padding) {
    // a padded substep (dt = 0): nothing to count, the loop stays done
    c->padded += 1;
    c->padding = 0;
    if (a.use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond_handle, 0u);
  } else if (threadIdx.x == 0) {
    c->PhysicalTime += c->dt;
    c->substeps += 1;
    int done = !(c->dtemp < 0.999999999 * c->DT);
    if (c->err) done = 1;
    if (c->nsub_dt >= FARGO_MAX_SUBSTEPS_PER_DT) {
      c->err |= FARGO_DEVERR_CAP;
      done = 1;
    }
    c->done = done;
    if (a.use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)a.cond_handle, done ? 0u : 1u);
  }
}
FARGO_F64_BODY(end_body)
template <class T>
__global__ void __launch_bounds__(256) k_end(const __grid_constant__ KArgs<T> a) {
  pdl_enter();
  FARGO_RUN_BODY(T, end_body, a, FARGO_BID);
}

// Start of a DT (AlgoGas entry, src/SourceEuler.cu:202-221).
__device__ __forceinline__ void dt_begin_body(Ctl *c) {
  c->dtemp = 0.0;
  c->nsub_dt = 0;
  c->done = 0;
  c->err = 0;
  c->ticket = 0u;
  c->padding = 0;
  c->ring_max[0] = c->ring_max[1] = FARGO_RING_NO_LIMIT;
}
__global__ void k_dt_begin(Ctl *c) {
  pdl_enter();
  dt_begin_body(c);
}

// ---------------------------------------------------------------------------
// Fused ensembles (fargo_batch_fuse): one launch of each substep kernel for a
// group of disks.  Member g of a group owns the launch's blocks first[g] ..
// first[g+1]-1, its own grid laid out gx[g] blocks wide; a block reads its disk and
// its place in that disk's grid from a per-block table, skips it when that disk's DT is over (masked subcycling: every
// disk keeps its own CFL step and substep count, and the loop runs until the last
// disk is done), and runs the kernel body of the single-disk launch with the
// disk's arguments and its own block index.
template <class T>
__device__ __forceinline__ const KArgs<T> *batch_block(const BatchGroup<T> &G, uint3 &bid, bool masked = true,
                                                       int *count = nullptr) {
  const int4 r = __ldg(&G.blk[blockIdx.x]);
  const KArgs<T> *a = &G.args[r.x & 0xFFFFF];
  if (masked && a->d.ctl->done) return nullptr;
  bid = make_uint3((unsigned)r.y, (unsigned)r.z, (unsigned)r.w);
  if (count) *count = r.x >> 20;
  return a;
}

// The body reads the disk's arguments in place (for T = double through the
// out-of-line body shared with the single-disk kernel).  (Copying them into
// shared memory first measured 5% faster on the 64-disk ensemble but changed the
// last bits of the inlined FP32 bodies against the single-disk kernels.)  A
// launched block may cover several consecutive blocks of its disk's grid along x
// (the per-cell kernels: the table read and the done test are paid once for all
// of them).
#define FARGO_BATCHED(kname, bounds, body, ...)                                  \
  template <class T>                                                             \
  __global__ void __launch_bounds__(bounds) kname(BatchGroup<T> G) {             \
    pdl_enter();                                                                 \
    uint3 bid;                                                                   \
    int cnt = 1;                                                                 \
    const KArgs<T> *a = batch_block(G, bid, true, &cnt);                         \
    if (!a) return;                                                              \
    for (int k = 0; k < cnt; k++) {                                              \
      const uint3 b = make_uint3(bid.x + k, bid.y, bid.z);                       \
      if constexpr (sizeof(T) == 8)                                              \
        body##_f64(*a, b, ##__VA_ARGS__);                                        \
      else                                                                       \
        body<T>(*a, b, ##__VA_ARGS__);                                           \
    }                                                                            \
  }
FARGO_BATCHED(kb_soundspeed, 256, soundspeed_body)
FARGO_BATCHED(kb_correct_vtheta, 256, correct_vtheta_body)
FARGO_BATCHED(kb_source, 256, source_body)
FARGO_BATCHED(kb_visc_tau, 256, visc_tau_body, G.extra ? a->d.vrad : a->d.vradint,
              G.extra ? a->d.vtheta : a->d.vthetaint)
FARGO_BATCHED(kb_visc_update, 256, visc_update_body)
FARGO_BATCHED(kb_artvisc, 256, artvisc_body)
FARGO_BATCHED(kb_energy, 256, energy_body)
FARGO_BATCHED(kb_velocities, 256, velocities_body, G.extra)
FARGO_BATCHED(kb_end, 256, end_body)
template <class T>
__global__ void __launch_bounds__(32 * RAD_NY) kb_radial(BatchGroup<T> G) {
  pdl_enter();
  uint3 bid;
  const KArgs<T> *ap = batch_block(G, bid);
  if (!ap) return;
  radial_body<T>(*ap, bid);
}
FARGO_BATCHED(kb_radial_col, RADC_THREADS, radial_col_body)
template <class T>
__global__ void __launch_bounds__(64) kb_planets(BatchGroup<T> G) {
  pdl_enter();
  uint3 bid;
  const KArgs<T> *ap = batch_block(G, bid);
  if (!ap) return;
  planets_body(ap->P, ap->d.ctl, ap->d.ring_force, sizeof(T) == 4);
}
#undef FARGO_BATCHED

template <class T, int V4>
__global__ void __launch_bounds__(256, V4 ? 1 : 2) kb_cfl_forces(BatchGroup<T> G) {
  pdl_enter();
  uint3 bid;
  const KArgs<T> *ap = batch_block(G, bid);
  if (!ap) return;
  cfl_forces_run<T, V4>(*ap, bid);
}
template <class T, bool MC>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 512 : 768) kb_azimuthal4(BatchGroup<T> G) {
  pdl_enter();
  uint3 bid;
  const KArgs<T> *ap = batch_block(G, bid);
  if (!ap) return;
  azimuthal4_run<T, MC>(*ap, bid);
}
// the start of a DT on every member (not masked: it clears the done flag)
template <class T>
__global__ void kb_dt_begin(BatchGroup<T> G) {
  pdl_enter();
  uint3 bid;
  const KArgs<T> *a = batch_block(G, bid, false);
  if (threadIdx.x == 0) dt_begin_body(a->d.ctl);
}
// the condition of the fused DT loop: another substep while any disk is not done
__global__ void kb_loop_cond(Ctl *const *ctls, int n, unsigned long long handle) {
  pdl_enter();
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int k = threadIdx.x; k < n; k += blockDim.x)
    if (!ctls[k]->done) any = 1;
  __syncthreads();
  if (threadIdx.x == 0) cudaGraphSetConditional((cudaGraphConditionalHandle)handle, any ? 1u : 0u);
}

template <class T>
void launch_batched(int kernel, const BatchGroup<T> &G, int nblocks, dim3 block, size_t smem, int pdl,
                    cudaStream_t s) {
  const dim3 g(nblocks);
  switch (kernel) {
    case BK_DT_BEGIN: launch_k(pdl, kb_dt_begin<T>, g, block, smem, s, G); probe_mark(s, "kb_dt_begin"); break;
    case BK_SOUNDSPEED: launch_k(pdl, kb_soundspeed<T>, g, block, smem, s, G); probe_mark(s, "kb_soundspeed"); break;
    case BK_CFL_V4: launch_k(pdl, kb_cfl_forces<T, 1>, g, block, smem, s, G); probe_mark(s, "kb_cfl_forces"); break;
    case BK_CFL: launch_k(pdl, kb_cfl_forces<T, 0>, g, block, smem, s, G); probe_mark(s, "kb_cfl_forces"); break;
    case BK_PLANETS: launch_k(pdl, kb_planets<T>, g, block, smem, s, G); probe_mark(s, "kb_planets"); break;
    case BK_COROT: launch_k(pdl, kb_correct_vtheta<T>, g, block, smem, s, G); probe_mark(s, "kb_correct_vtheta"); break;
    case BK_SOURCE: launch_k(pdl, kb_source<T>, g, block, smem, s, G); probe_mark(s, "kb_source"); break;
    case BK_VISC_TAU: launch_k(pdl, kb_visc_tau<T>, g, block, smem, s, G); probe_mark(s, "kb_visc_tau"); break;
    case BK_VISC_UPDATE: launch_k(pdl, kb_visc_update<T>, g, block, smem, s, G); probe_mark(s, "kb_visc_update"); break;
    case BK_ARTVISC: launch_k(pdl, kb_artvisc<T>, g, block, smem, s, G); probe_mark(s, "kb_artvisc"); break;
    case BK_ENERGY: launch_k(pdl, kb_energy<T>, g, block, smem, s, G); probe_mark(s, "kb_energy"); break;
    case BK_RADIAL: launch_k(pdl, kb_radial<T>, g, block, smem, s, G); probe_mark(s, "kb_radial"); break;
    case BK_RADIAL_COL: launch_k(pdl, kb_radial_col<T>, g, block, smem, s, G); probe_mark(s, "kb_radial_col"); break;
    case BK_AZ4: launch_k(pdl, kb_azimuthal4<T, false>, g, block, smem, s, G); probe_mark(s, "kb_azimuthal4"); break;
    case BK_AZ4_MC: launch_k(pdl, kb_azimuthal4<T, true>, g, block, smem, s, G); probe_mark(s, "kb_azimuthal4"); break;
    case BK_VELOCITIES: launch_k(pdl, kb_velocities<T>, g, block, smem, s, G); probe_mark(s, "kb_velocities"); break;
    case BK_END: launch_k(pdl, kb_end<T>, g, block, smem, s, G); probe_mark(s, "kb_end"); break;
    default: break;
  }
}

void launch_loop_cond(Ctl *const *ctls, int n, unsigned long long handle, int pdl, cudaStream_t s) {
  launch_k(pdl, kb_loop_cond, dim3(1), dim3(256), 0, s, ctls, n, handle);
  probe_mark(s, "kb_loop_cond");
}

// prepares the batched kernels that take more than 48 KB of shared memory
template <class T>
cudaError_t prepare_batched(size_t rad_smem, size_t az_smem) {
  cudaError_t e;
  const void *all[] = {(const void *)kb_dt_begin<T>, (const void *)kb_soundspeed<T>,
                       (const void *)kb_cfl_forces<T, 1>, (const void *)kb_cfl_forces<T, 0>,
                       (const void *)kb_planets<T>, (const void *)kb_correct_vtheta<T>, (const void *)kb_source<T>,
                       (const void *)kb_visc_tau<T>, (const void *)kb_visc_update<T>, (const void *)kb_artvisc<T>,
                       (const void *)kb_energy<T>, (const void *)kb_radial<T>, (const void *)kb_azimuthal4<T, false>,
                       (const void *)kb_azimuthal4<T, true>, (const void *)kb_velocities<T>, (const void *)kb_end<T>,
                       (const void *)kb_loop_cond};
  for (const void *f : all)
    if ((e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, FARGO_SMEM_CARVEOUT)) !=
        cudaSuccess)
      return e;
  if ((e = cudaFuncSetAttribute(kb_radial<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rad_smem)) !=
      cudaSuccess)
    return e;
  if (az_smem > 0) {
    if ((e = cudaFuncSetAttribute(kb_azimuthal4<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)az_smem)) != cudaSuccess)
      return e;
    if ((e = cudaFuncSetAttribute(kb_azimuthal4<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)az_smem)) != cudaSuccess)
      return e;
  }
  return cudaSuccess;
}

// ---------------------------------------------------------------------------
// host-side launchers.  MARK records the launch in the optional probe (launch
// counting, per-kernel CUDA-event timing); it never changes what runs.
thread_local LaunchProbe *g_probe = nullptr;
#define MARK(name) probe_mark(s, name)

template <class T>
void launch_substep_kernels(const KArgs<T> &a0, cudaStream_t s, unsigned which_mask, size_t az_smem_bytes,
                            const SideBranch *side, unsigned rot) {
  KArgs<T> a = a0;
  const DevParams &P = a.P;
  const dim3 b2(a.cell_bx, a.cell_by);
  const dim3 g2((P.nsec + a.cell_bx - 1) / a.cell_bx, (P.nrad + a.cell_by - 1) / a.cell_by);
  bool joined = true;
  const bool head_done = rot & ROT_HEAD_DONE;
  const bool bc1 = (which_mask & SUBK_BC1) && (P.open_inner || P.non_reflecting || P.evanescent);
  const bool sg_side =
      !head_done && side && (which_mask & SUBK_SG) && P.self_gravity && (which_mask & SUBK_CFL_FORCES) && !bc1;
  const bool sg_ahead = sg_side && (rot & SG_AHEAD) && (which_mask & SUBK_TRANSPORT);
  if (!head_done) {
    // the fork point precedes k_cfl_forces; the transforms are issued after it
    // (the earlier-issued grid is scheduled first, and the CFL kernel is the longer)
    if (sg_side) cudaEventRecord(side->fork2, s);
    if (which_mask & SUBK_CFL_FORCES) {
      // a.mode: 0 CFL + forces + planets, 2 forces + planets with dt = sloppy_dt,
      // 3 forces + potential only (no planet advance, no time update)
      launch_cfl_forces(a, s);
      MARK("k_cfl_forces");
    }
    if (sg_side) {
      cudaStreamWaitEvent(side->s2, side->fork2, 0);
      if (sg_ahead) launch_sg_cols_inv(a, side->s2);
      else launch_selfgravity(a, side->s2);
      cudaEventRecord(side->join2, side->s2);
    }
  }
  if (which_mask & SUBK_CFL_FORCES) {
    if (a.mode == 0 || a.mode == 2) {
      if (side && !P.corotating) {
        cudaEventRecord(side->fork, s);
        cudaStreamWaitEvent(side->s, side->fork, 0);
        k_planets<<<1, 64, 0, side->s>>>(P, a.d.ctl, a.d.ring_force, sizeof(T) == 4);
        cudaEventRecord(side->join, side->s);
        joined = false;
        if (g_probe) g_probe->count++;
      } else {
        k_planets<<<1, 64, 0, s>>>(P, a.d.ctl, a.d.ring_force, sizeof(T) == 4);
        MARK("k_planets");
      }
    }
  }
  if ((which_mask & SUBK_COROT) && P.corotating) {
    launch_k(a.pdl, k_correct_vtheta<T>, dim3(g2), dim3(b2), 0, s, a);
    MARK("k_correct_vtheta");
  }
  if (which_mask & SUBK_BC1) launch_boundaries(a, s);
  if ((which_mask & SUBK_SG) && P.self_gravity && !head_done) {
    if (sg_side) cudaStreamWaitEvent(s, side->join2, 0);
    else launch_selfgravity(a, s);
  }
  if (which_mask & SUBK_SOURCE) {
    launch_k(a.pdl, k_source<T>, dim3(g2), dim3(b2), 0, s, a);
    MARK("k_source");
    launch_k(a.pdl, k_visc_tau<T>, dim3(g2), dim3(b2), 0, s, a, a.d.vradint, a.d.vthetaint);
    MARK("k_visc_tau");
    launch_k(a.pdl, k_visc_update<T>, dim3(g2), dim3(b2), 0, s, a);
    MARK("k_visc_update");
    launch_k(a.pdl, k_artvisc<T>, dim3(g2), dim3(b2), 0, s, a);
    MARK("k_artvisc");
  }
  if (which_mask & SUBK_BC2) launch_boundaries(a, s);
  if ((which_mask & SUBK_ENERGY) && P.adiabatic) {
    // the viscous stresses of the new velocities are formed inside k_energy
    launch_k(a.pdl, k_energy<T>, dim3(g2), dim3(b2), 0, s, a);
    MARK("k_energy");
  }
  const bool bc = P.open_inner || P.non_reflecting || P.evanescent;
  if (which_mask & SUBK_TRANSPORT) {
    if (a.rad_col) {
      launch_k(a.pdl, k_transport_radial_col<T>,
               dim3((P.nsec + RADC_THREADS - 1) / RADC_THREADS, (P.nrad + RADC_RINGS - 1) / RADC_RINGS),
               dim3(RADC_THREADS), 0, s, a);
      MARK("k_transport_radial_col");
    } else if (a.rad_maps) {
      launch_k(a.pdl, k_transport_radial_tma<T>, dim3(a.rad_grid), dim3(32, RAD_NY), RAD_TMA_SMEM(T), s, a,
               *a.rad_maps);
      MARK("k_transport_radial_tma");
    } else {
      launch_k(a.pdl, k_transport_radial<T>, dim3((P.nsec + 31) / 32, (P.nrad + RAD_TR - 1) / RAD_TR),
               dim3(32, RAD_NY), RAD_SMEM(T), s, a);
      MARK("k_transport_radial");
    }
    if (a.az_regs) {
      // one chunk of four cells per thread up to the CTA's size, or (az_chunks = 2)
      // half the threads with two chunks each
      const int nt4 = az4_threads<T>(a.az_chunks == 2 ? P.nsec / 2 : P.nsec);
      if (P.nsec / 4 > nt4)
        launch_k(a.pdl, k_transport_azimuthal4<T, true>, dim3(P.nrad), dim3(nt4), az_smem_bytes, s, a);
      else
        launch_k(a.pdl, k_transport_azimuthal4<T, false>, dim3(P.nrad), dim3(nt4), az_smem_bytes, s, a);
    } else {
      int nt = P.nsec >= 1024 ? 512 : 256;
      a.az_smem = az_smem_bytes > 0;
      launch_k(a.pdl, k_transport_azimuthal<T>, dim3(P.nrad), dim3(nt), az_smem_bytes, s, a);
      a.az_smem = 0;
    }
    MARK("k_transport_azimuthal");
    if (sg_ahead) {
      // the next substep's ring transforms, from the final density, beside the
      // velocities and k_end (the DT's last substep's are unused: the DT prefix
      // transforms the density it starts from)
      cudaEventRecord(side->fork2, s);
      cudaStreamWaitEvent(side->s2, side->fork2, 0);
      launch_sg_rows_fwd(a, side->s2);
      cudaEventRecord(side->join2, side->s2);
    }
    launch_k(a.pdl, k_velocities<T>, dim3(g2), dim3(b2), 0, s, a, (!bc && (which_mask & SUBK_TEMPERATURE)) ? 1 : 0);
    MARK("k_velocities");
  }
  if (which_mask & SUBK_BC3) launch_boundaries(a, s);
  if ((which_mask & SUBK_TEMPERATURE) && (bc || !(which_mask & SUBK_TRANSPORT))) {
    launch_k(a.pdl, k_temperature<T>, dim3(g2), dim3(b2), 0, s, a);
    MARK("k_temperature");
  }
  if (which_mask & SUBK_END) {
    launch_k(a.pdl, k_end<T>, dim3(1), dim3(256), 0, s, a);
    MARK("k_end");
  }
  if (rot & ROT_NEXT_HEAD) {
    // the next substep's transforms (they read only the density, final now) beside
    // its CFL/force kernel; both return at once when this substep ended the DT
    // (the loop flag k_end just set, which nothing else writes before the next k_end)
    cudaEventRecord(side->fork2, s);
    cudaStreamWaitEvent(side->s2, side->fork2, 0);
    KArgs<T> g2s = a;
    g2s.guard = 1;
    launch_selfgravity(g2s, side->s2);
    cudaEventRecord(side->join2, side->s2);
    // the next substep's CFL/force kernel, after this substep's planet update
    // (it reads the planet parameters that update leaves)
    if (!joined) {
      cudaStreamWaitEvent(s, side->join, 0);
      joined = true;
    }
    KArgs<T> g = a;
    g.guard = 1;
    launch_cfl_forces(g, s);
    MARK("k_cfl_forces");
    cudaStreamWaitEvent(s, side->join2, 0);
  }
  if (!joined) cudaStreamWaitEvent(s, side->join, 0);
  if (sg_ahead) cudaStreamWaitEvent(s, side->join2, 0);
}

// The first substep's CFL/force kernel and self-gravity transforms, side by side,
// ahead of a DT loop whose substeps launch the next substep's (ROT_NEXT_HEAD).
template <class T>
void launch_dt_head(const KArgs<T> &a, cudaStream_t s, const SideBranch *side) {
  cudaEventRecord(side->fork2, s);
  launch_cfl_forces(a, s);
  MARK("k_cfl_forces");
  cudaStreamWaitEvent(side->s2, side->fork2, 0);
  launch_selfgravity(a, side->s2);
  cudaEventRecord(side->join2, side->s2);
  cudaStreamWaitEvent(s, side->join2, 0);
}

// whether a DT loop may run rotated: self-gravity, no boundary kernel that
// changes the density, side streams available
template <class T>
bool rotation_allowed(const KArgs<T> &a, const SideBranch *side) {
  const DevParams &P = a.P;
  return side && P.self_gravity && !(P.open_inner || P.non_reflecting || P.evanescent);
}

// whether a DT loop may run its ring transforms ahead (SG_AHEAD): the same
// conditions as the rotated loop
template <class T>
bool sg_ahead_allowed(const KArgs<T> &a, const SideBranch *side) {
  return rotation_allowed(a, side);
}

template <class T>
void launch_boundaries(const KArgs<T> &a, cudaStream_t s) {
  const DevParams &P = a.P;
  if (P.open_inner) {
    launch_k(a.pdl, k_bc_open<T>, dim3((P.nsec + 255) / 256), dim3(256), 0, s, a);
    MARK("k_bc_open");
  }
  if (P.non_reflecting) {
    if (P.adiabatic) {
      launch_k(a.pdl, k_soundspeed<T>, dim3(P.nrad), dim3(256), 0, s, a);
      MARK("k_soundspeed");
    }
    const dim3 gj((P.nsec + 255) / 256);
    launch_k(a.pdl, k_bc_nr_means<T>, dim3(4), dim3(256), 0, s, a, 0);
    MARK("k_bc_nr_means");
    launch_k(a.pdl, k_bc_nr_cells<T>, gj, dim3(256), 0, s, a);
    MARK("k_bc_nr_cells");
    launch_k(a.pdl, k_bc_nr_means<T>, dim3(4), dim3(256), 0, s, a, 1);
    MARK("k_bc_nr_means");
    launch_k(a.pdl, k_bc_nr_adjust<T>, gj, dim3(256), 0, s, a);
    MARK("k_bc_nr_adjust");
  }
  if (P.evanescent) {
    const dim3 b2(a.cell_bx, a.cell_by);
    const dim3 g2((P.nsec + a.cell_bx - 1) / a.cell_bx, (P.nrad + a.cell_by - 1) / a.cell_by);
    launch_k(a.pdl, k_bc_evanescent<T>, dim3(g2), dim3(b2), 0, s, a);
    MARK("k_bc_evanescent");
  }
}

template <class T>
void launch_dt_prefix(const KArgs<T> &a0, cudaStream_t s) {
  KArgs<T> a = a0;
  launch_k(a.pdl, k_dt_begin, dim3(1), dim3(1), 0, s, a.d.ctl);
  MARK("k_dt_begin");
  if (a.P.adiabatic) {
    launch_k(a.pdl, k_soundspeed<T>, dim3(a.P.nrad), dim3(256), 0, s, a);
    MARK("k_soundspeed");
  }
  if (a.P.sloppy_cfl) {
    a.mode = 1;
    launch_cfl_forces(a, s);
    MARK("k_cfl_forces");
  }
}

template <class T>
void launch_cfl_only(const KArgs<T> &a0, cudaStream_t s) {
  KArgs<T> a = a0;
  a.mode = 1;
  launch_cfl_forces(a, s);
  MARK("k_cfl_forces");
}

template <class T>
int rad_tma_grid(int nrad, int nsec) {
  int dev = 0, sms = 0, per = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_transport_radial_tma<T>, 32 * RAD_NY,
                                                    RAD_TMA_SMEM(T)) != cudaSuccess || per < 1)
    return 0;
  const int tiles = ((nsec + 31) / 32) * ((nrad + RAD_TR - 1) / RAD_TR);
  return tiles < sms * per ? tiles : sms * per;
}

template <class T>
cudaError_t prepare_kernels(size_t az_smem_bytes, int az_regs) {
  // One shared-memory carveout for every step kernel: an SM changes its L1 /
  // shared split only when idle, so kernels that run side by side (the CFL/force
  // kernel, the self-gravity transforms, the planet update) and successive
  // kernels under programmatic launch can share SMs only with the same split.
  const void *all[] = {(const void *)k_cfl_forces<T, 0>, (const void *)k_cfl_forces<T, 1>, (const void *)k_planets, (const void *)k_soundspeed<T>,
                       (const void *)k_correct_vtheta<T>, (const void *)k_bc_open<T>,
                       (const void *)k_bc_nr_means<T>, (const void *)k_bc_nr_cells<T>,
                       (const void *)k_bc_nr_adjust<T>, (const void *)k_bc_evanescent<T>,
                       (const void *)k_source<T>, (const void *)k_visc_tau<T>, (const void *)k_visc_update<T>,
                       (const void *)k_artvisc<T>, (const void *)k_energy<T>, (const void *)k_transport_radial<T>,
                       (const void *)k_transport_azimuthal<T>, (const void *)k_transport_azimuthal4<T, false>,
                       (const void *)k_transport_azimuthal4<T, true>,
                       (const void *)k_velocities<T>, (const void *)k_temperature<T>, (const void *)k_end<T>,
                       (const void *)k_dt_begin};
  cudaError_t e;
  for (const void *f : all)
    if ((e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout, FARGO_SMEM_CARVEOUT)) != cudaSuccess)
      return e;
  e = cudaFuncSetAttribute(k_transport_radial<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RAD_SMEM(T));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_transport_radial_tma<T>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           FARGO_SMEM_CARVEOUT);
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(k_transport_radial_tma<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)RAD_TMA_SMEM(T));
  if (e != cudaSuccess) return e;
  if (az_smem_bytes == 0) return cudaSuccess;
  if (az_regs) {
    e = cudaFuncSetAttribute(k_transport_azimuthal4<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)az_smem_bytes);
    if (e != cudaSuccess) return e;
    return cudaFuncSetAttribute(k_transport_azimuthal4<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)az_smem_bytes);
  }
  return cudaFuncSetAttribute(k_transport_azimuthal<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)az_smem_bytes);
}

// FP64 host data <-> device fields of type T through an FP64 staging buffer
template <class T>
__global__ void k_convert_from_f64(const double *__restrict__ in, T *__restrict__ out, size_t n) {
  pdl_enter();
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    out[k] = (T)in[k];
}
template <class T>
__global__ void k_convert_to_f64(const T *__restrict__ in, double *__restrict__ out, size_t n) {
  pdl_enter();
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    out[k] = (double)in[k];
}
// Several fields in one launch (the fields of one host transfer)
template <class T>
__global__ void k_convert_from_f64_multi(ConvFields p, size_t n) {
  pdl_enter();
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    for (int f = 0; f < p.nf; f++) ((T *)p.dst[f])[k] = (T)((const double *)p.src[f])[k];
}
template <class T>
__global__ void k_convert_to_f64_multi(ConvFields p, size_t n) {
  pdl_enter();
  for (size_t k = blockIdx.x * (size_t)blockDim.x + threadIdx.x; k < n; k += (size_t)gridDim.x * blockDim.x)
    for (int f = 0; f < p.nf; f++) ((double *)p.dst[f])[k] = (double)((const T *)p.src[f])[k];
}
void launch_convert_from_f64_multi(const ConvFields &p, size_t n, int esize, cudaStream_t s) {
  if (esize == 4) k_convert_from_f64_multi<float><<<608, 256, 0, s>>>(p, n);
  else k_convert_from_f64_multi<double><<<608, 256, 0, s>>>(p, n);
}
void launch_convert_to_f64_multi(const ConvFields &p, size_t n, int esize, cudaStream_t s) {
  if (esize == 4) k_convert_to_f64_multi<float><<<608, 256, 0, s>>>(p, n);
  else k_convert_to_f64_multi<double><<<608, 256, 0, s>>>(p, n);
}
void launch_convert_from_f64(const double *in, void *out, size_t n, int esize, cudaStream_t s) {
  if (esize == 4) k_convert_from_f64<float><<<608, 256, 0, s>>>(in, (float *)out, n);
  else k_convert_from_f64<double><<<608, 256, 0, s>>>(in, (double *)out, n);
}
void launch_convert_to_f64(const void *in, double *out, size_t n, int esize, cudaStream_t s) {
  if (esize == 4) k_convert_to_f64<float><<<608, 256, 0, s>>>((const float *)in, out, n);
  else k_convert_to_f64<double><<<608, 256, 0, s>>>((const double *)in, out, n);
}

#define INSTANTIATE(T)                                                                                  \
  template void launch_substep_kernels<T>(const KArgs<T> &, cudaStream_t, unsigned, size_t,            \
                                         const SideBranch *, unsigned);                                \
  template void launch_dt_head<T>(const KArgs<T> &, cudaStream_t, const SideBranch *);                  \
  template bool sg_ahead_allowed<T>(const KArgs<T> &, const SideBranch *);                            \
  template bool rotation_allowed<T>(const KArgs<T> &, const SideBranch *);                              \
  template void launch_dt_prefix<T>(const KArgs<T> &, cudaStream_t);                                    \
  template void launch_cfl_only<T>(const KArgs<T> &, cudaStream_t);                                     \
  template void launch_boundaries<T>(const KArgs<T> &, cudaStream_t);                                   \
  template cudaError_t prepare_kernels<T>(size_t, int); \
  template int rad_tma_grid<T>(int, int);                                                              \
  template void launch_batched<T>(int, const BatchGroup<T> &, int, dim3, size_t, int, cudaStream_t);   \
  template cudaError_t prepare_batched<T>(size_t, size_t);                                                \
  template int az4_threads_host<T>(int);
INSTANTIATE(double)
INSTANTIATE(float)
