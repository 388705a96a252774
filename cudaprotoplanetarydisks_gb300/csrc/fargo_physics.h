// fargo_physics.h -- shared host/device definitions of the step's small FP64 parts.
//
// DevParams: the parameter set as kernels see it (by value).
// Ctl: the per-context control block that lives in device memory; it carries
// the time state, the CFL decision, the planetary system and the per-substep
// scalars from kernel to kernel, so a whole DT runs without the host.
// The FARGO_HD functions restate the reference's scalar host code (planet
// integration, frame rotation, profiles) and run on the host at set-up and on
// one device thread inside the step.  All FP64 in every precision mode.
#pragma once

#include <math.h>

#if defined(__CUDACC__)
#define FARGO_HD __host__ __device__ inline
#else
#define FARGO_HD inline
#endif

#define FARGO_MAXPL 16
#define FARGO_PI 3.14159265358979323844  /* include/Fondam.cuh:4 */
#define FARGO_CFLSECURITY 0.5            /* include/Fondam.cuh:7 */
#define FARGO_CVNR 1.41                  /* include/Fondam.cuh:10 */
#define FARGO_MAX_SUBSTEPS_PER_DT 100000

// error bits set on the device
#define FARGO_DEVERR_CFL 1        // non-finite or non-positive CFL time step
#define FARGO_DEVERR_CAP 2        // too many substeps in one DT
#define FARGO_DEVERR_NAN 4        // non-finite density found
#define FARGO_DEVERR_WAIT 8       // a bounded wait on an asynchronous copy gave up

struct DevParams {
  int nrad, nsec, nb, nsec2pot;
  int adiabatic, cooling, self_gravity, fast_transport;
  int open_inner, non_reflecting, evanescent, corotating, guiding_center;
  int indirect_term, exclude_hill, viscosity_alpha, roche_smoothing, forced_circular;
  int sloppy_cfl, is_disk;
  int nu_dynamic;   // recompute the viscosity profile on the device each substep
  double DT;
  double aspectratio, flaringindex, sigmaslope, sigma0, imposeddiskdrift;
  double adiabaticindex, coolingtime0;
  double thicknesssmoothing, rochesmoothing, masstaper, releaseradius, releasedate;
  double transitionradius, transitionratio, transitionwidth, lambdadoubling;
  double viscosity, alphaviscosity, cavityradius, cavityratio, cavitywidth;
  double sgp_eps, sgp_rstep, sgp_tstep;
};

// "No limit" of a per-ring time step: a NaN bit pattern, above every non-negative
// double (+inf included) when compared as a signed 64-bit integer.
#define FARGO_RING_NO_LIMIT 0LL  // the bit pattern of +0.0: no ring has a limit

struct Ctl {
  // time state (reference globals PhysicalTime, OmegaFrame, LostMass; AlgoGas locals)
  double DT, dtemp, dt;
  double PhysicalTime, PhysicalTimeInitial, OmegaFrame, MassTaper, domega;
  double LostMass;
  double ind_x, ind_y;        // IndirectTerm (Pframeforce.cu:24)
  double sloppy_dt;
  int cfl, done, err, nsub_dt;
  long long substeps;
  unsigned int ticket;        // last-block-done counter of the CFL/force kernel
  int padding;                // 1: the running substep pads the loop body (dt = 0)
  // largest per-ring S (sum of squared inverse time steps) and angular-velocity
  // difference of the CFL/force kernel, as the integers of their (positive) bit
  // patterns; FARGO_RING_NO_LIMIT between launches
  long long ring_max[2];
  // dt of the last substep that advanced the disk (a padded substep runs with
  // dt = 0), and the number of padded substeps run
  double dt_sub;
  long long padded;
  // ring means of the non-reflecting boundary: sound speed of rings 0, 1, nrad-1,
  // nrad-2, then density and energy of rings 0 and nrad-1 after the shift
  double bc_mean[8];
  // planetary system (Types.cuh:2-12)
  int nb;
  int pad1;
  double x[FARGO_MAXPL], y[FARGO_MAXPL], vx[FARGO_MAXPL], vy[FARGO_MAXPL];
  double mass[FARGO_MAXPL], acc[FARGO_MAXPL];
  int feeldisk[FARGO_MAXPL], feelothers[FARGO_MAXPL];
  // GetPsysInfo statics (Psys.cu:79)
  double xmark, ymark;
  // per-substep planet parameters, computed once after each planet update:
  // bodies feeling the disk (0 = the star) and the potential of every planet
  int nbody;
  int pad2;
  double bx[FARGO_MAXPL + 1], by[FARGO_MAXPL + 1], brs2[FARGO_MAXPL + 1];
  double px[FARGO_MAXPL], py[FARGO_MAXPL], pm[FARGO_MAXPL], ps2[FARGO_MAXPL], pinvd3[FARGO_MAXPL];
  // disk accelerations of the bodies (ComputeAccel) and start time of the substep
  double accx[FARGO_MAXPL + 1], accy[FARGO_MAXPL + 1];
  double t_sub;
  // FP32 copies of the per-substep scalars the field kernels read (CTL_F_*), so
  // that FP32 kernels convert nothing per thread; refreshed with their FP64 values
  float f32[8];
};

enum { CTL_F_DT = 0, CTL_F_OMEGA, CTL_F_INDX, CTL_F_INDY, CTL_F_DOMEGA, CTL_F_INVDT, CTL_F_COUNT };

// refresh every FP32 copy from its FP64 value
FARGO_HD void fargo_ctl_mirror(Ctl &c) {
  c.f32[CTL_F_DT] = (float)c.dt;
  c.f32[CTL_F_OMEGA] = (float)c.OmegaFrame;
  c.f32[CTL_F_INDX] = (float)c.ind_x;
  c.f32[CTL_F_INDY] = (float)c.ind_y;
  c.f32[CTL_F_DOMEGA] = (float)c.domega;
  c.f32[CTL_F_INVDT] = c.dt != 0.0 ? 1.0f / (float)c.dt : 0.0f;
  c.ring_max[0] = c.ring_max[1] = FARGO_RING_NO_LIMIT;
}

// AspectRatioHost / AspectRatioDevice  src/Viscosity.cu:93-107, src/Kernels.cu:1377-1392
FARGO_HD double fargo_aspect_ratio(const DevParams &P, double r, double t, double t0) {
  double aspectratio, rmin, rmax, scale;
  aspectratio = P.aspectratio;
  rmin = P.transitionradius - P.transitionwidth * P.aspectratio;
  rmax = P.transitionradius + P.transitionwidth * P.aspectratio;
  scale = 1.0 + (t - t0) * P.lambdadoubling;
  rmin *= scale;
  rmax *= scale;
  if (r < rmin) aspectratio *= P.transitionratio;
  if ((r >= rmin) && (r <= rmax)) aspectratio *= exp((rmax - r) / (rmax - rmin) * log(P.transitionratio));
  return aspectratio;
}

// The cavity factor of FViscosity (src/Viscosity.cu:40-48): cavityratio inside the
// cavity, an exponential ramp across its edge, 1 outside.
FARGO_HD double fargo_cavity_factor(const DevParams &P, double r, double t, double t0) {
  double rmin, rmax, scale;
  rmin = P.cavityradius - P.cavitywidth * P.aspectratio;
  rmax = P.cavityradius + P.cavitywidth * P.aspectratio;
  scale = 1.0 + (t - t0) * P.lambdadoubling;
  rmin *= scale;
  rmax *= scale;
  if (r < rmin) return P.cavityratio;
  if ((r >= rmin) && (r <= rmax)) return exp((rmax - r) / (rmax - rmin) * log(P.cavityratio));
  return 1.0;
}

// FViscosity  src/Viscosity.cu:33-50; csmean is GLOBAL_bufarray[i] for r = Rmed[i].
// The cavity branches multiply once (by the factor above; a factor 1 is exact).
FARGO_HD double fargo_fviscosity(const DevParams &P, double r, double csmean, double t, double t0) {
  double viscosity = P.viscosity;
  if (P.viscosity_alpha) viscosity = P.alphaviscosity * csmean * csmean * pow(r, 1.5);
  return viscosity * fargo_cavity_factor(P, r, t, t0);
}

// pow with the exponents 0, 1 and 2 of the usual disk set-ups (flat flaring,
// squares) taken exactly: x^0 = 1, x^1 = x, x^2 = x*x are the correctly rounded
// powers, and an FP64 pow costs thousands of cycles on this GPU.
FARGO_HD double fargo_pow(double x, double e) {
  if (e == 1.0) return x;
  if (e == 2.0) return x * x;
  if (e == 0.0) return 1.0;
  return pow(x, e);
}

// Compute_smoothing  src/Force.cu:137-142
FARGO_HD double fargo_smoothing(const DevParams &P, double r, double t, double t0) {
  return P.thicknesssmoothing * fargo_aspect_ratio(P, r, t, t0) * fargo_pow(r, 1.0 + P.flaringindex);
}

// MassTaper  src/SourceEuler.cu:223-224
FARGO_HD double fargo_mass_taper(const DevParams &P, double t) {
  double m = t / (P.masstaper * 2.0 * M_PI);
  return (m > 1.0 ? 1.0 : fargo_pow(sin(m * M_PI / 2.0), 2.0));
}

// GetPsysInfo  src/Psys.cu:249-319 (action 0 = GET, 1 = MARK, 2 = FREQUENCY)
FARGO_HD double fargo_psys_info(Ctl &c, const DevParams &P, int action) {
  double d1, d2, cross, x, y, vx, vy, m, h, d, Ax, Ay, e, a, E, M, xc, yc, omega, arg, PerihelionPA;
  xc = x = c.x[0];
  yc = y = c.y[0];
  vx = c.vx[0];
  vy = c.vy[0];
  m = c.mass[0] + 1.;
  h = x * vy - y * vx;
  d = sqrt(x * x + y * y);
  Ax = x * vy * vy - y * vx * vy - 1.0 * m * x / d;
  Ay = y * vx * vx - x * vx * vy - 1.0 * m * y / d;
  e = sqrt(Ax * Ax + Ay * Ay) / m;
  a = h * h / 1.0 / m / (1. - e * e);
  if (e == 0.0) arg = 1.0;
  else arg = (1.0 - d / a) / e;
  if (fabs(arg) >= 1.0) E = FARGO_PI * (1. - arg / fabs(arg)) / 2.;
  else E = acos((1.0 - d / a) / e);
  if ((x * y * (vy * vy - vx * vx) + vx * vy * (x * x - y * y)) < 0) E = -E;
  M = E - e * sin(E);
  PerihelionPA = atan2(Ay, Ax);
  omega = sqrt(m / a / a / a);
  if (P.guiding_center) {
    xc = a * cos(M + PerihelionPA);
    yc = a * sin(M + PerihelionPA);
  }
  if (e < 1e-08) {
    xc = x;
    yc = y;
  }
  switch (action) {
    case 1:
      c.xmark = xc;
      c.ymark = yc;
      return 0.;
    case 0:
      x = xc;
      y = yc;
      d2 = sqrt(x * x + y * y);
      d1 = sqrt(c.xmark * c.xmark + c.ymark * c.ymark);
      cross = c.xmark * y - x * c.ymark;
      c.xmark = x;
      c.ymark = y;
      return asin(cross / (d1 * d2));
    case 2:
      return omega;
  }
  return 0.0;
}

// RotatePsys  src/Psys.cu:323-340 (rotate by -angle)
FARGO_HD void fargo_rotate_psys(Ctl &c, double angle) {
  // sin 0 = 0 and cos 0 = 1 exactly: a fixed frame skips the two FP64 calls
  double sint = 0.0, cost = 1.0;
  if (angle != 0.0) {
    sint = sin(angle);
    cost = cos(angle);
  }
  for (int i = 0; i < c.nb; i++) {
    double xt = c.x[i], yt = c.y[i];
    c.x[i] = xt * cost + yt * sint;
    c.y[i] = -xt * sint + yt * cost;
    xt = c.vx[i];
    yt = c.vy[i];
    c.vx[i] = xt * cost + yt * sint;
    c.vy[i] = -xt * sint + yt * cost;
  }
}

// DerivMotionRK5  src/RungeKutta.cu:30-67 (the feel-others term uses the
// distance of body j to the star, as the reference does).  NB > 0: NB bodies,
// a compile-time count that keeps every array in registers; NB == 0: nb bodies.
template <int NB>
FARGO_HD void fargo_deriv_rk5(const double *q, const double *pm, double *deriv, int nb_rt, double dt,
                              const int *feelothers, int indirect) {
  const int nb = NB > 0 ? NB : nb_rt;
  const double *x = q, *y = x + nb, *vx = y + nb, *vy = vx + nb;
  double *dx = deriv, *dy = dx + nb, *dvx = dy + nb, *dvy = dvx + nb;
  // 1/d^3 of each body with one divide (the reference divides three times; an
  // FP64 divide is a long dependent sequence on this GPU's FP64 pipe)
  double Inv3[NB > 0 ? NB : FARGO_MAXPL];
#pragma unroll
  for (int i = 0; i < nb; i++) {
    const double d = sqrt(x[i] * x[i] + y[i] * y[i]);
    Inv3[i] = 1.0 / (d * d * d);
  }
#pragma unroll
  for (int i = 0; i < nb; i++) {
    dx[i] = vx[i];
    dy[i] = vy[i];
    dvx[i] = -1.0 * Inv3[i] * x[i];
    dvy[i] = -1.0 * Inv3[i] * y[i];
#pragma unroll
    for (int j = 0; j < nb; j++) {
      if (indirect) {
        dvx[i] -= 1.0 * pm[j] * Inv3[j] * x[j];
        dvy[i] -= 1.0 * pm[j] * Inv3[j] * y[j];
      }
      if ((j != i) && (feelothers[i] == 1)) {
        dvx[i] += 1.0 * pm[j] * Inv3[j] * (x[j] - x[i]);
        dvy[i] += 1.0 * pm[j] * Inv3[j] * (y[j] - y[i]);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < 4 * nb; i++) deriv[i] *= dt;
}

// AdvanceSystemRK5's Cash-Karp step (src/RungeKutta.cu:70-130) from the state q0,
// result in q1; NB as for fargo_deriv_rk5.
template <int NB>
FARGO_HD void fargo_rk5_step(const double *q0, const double *pm, double *q1, int nb_rt, double dt,
                             const int *feelothers, int indirect) {
  constexpr int CAP = 4 * (NB > 0 ? NB : FARGO_MAXPL);
  const int nb = NB > 0 ? NB : nb_rt;
  double k[6][CAP];
#pragma unroll
  for (int s = 0; s < 6; s++)
#pragma unroll
    for (int i = 0; i < 4 * nb; i++) k[s][i] = 0.0;
  const double cf[5][5] = {{0.2, 0.0, 0.0, 0.0, 0.0},
                           {0.075, 0.225, 0.0, 0.0, 0.0},
                           {0.3, -0.9, 1.2, 0.0, 0.0},
                           {-11.0 / 54.0, 2.5, -70.0 / 27.0, 35.0 / 27.0, 0.0},
                           {1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0}};
  fargo_deriv_rk5<NB>(q0, pm, k[0], nb, dt, feelothers, indirect);
#pragma unroll
  for (int s = 0; s < 5; s++) {
#pragma unroll
    for (int i = 0; i < 4 * nb; i++)
      q1[i] = q0[i] + cf[s][0] * k[0][i] + cf[s][1] * k[1][i] + cf[s][2] * k[2][i] + cf[s][3] * k[3][i] +
              cf[s][4] * k[4][i];
    fargo_deriv_rk5<NB>(q1, pm, k[s + 1], nb, dt, feelothers, indirect);
  }
#pragma unroll
  for (int i = 0; i < 4 * nb; i++)
    q1[i] = q0[i] + 37.0 / 378.0 * k[0][i] + 250.0 / 621.0 * k[2][i] + 125.0 / 594.0 * k[3][i] +
            512.0 / 1771.0 * k[5][i];
}

// the step for nb bodies: one or two bodies (the usual set-ups) run a variant
// whose arrays live in registers, the same arithmetic
template <int NB>
FARGO_HD void fargo_rk5_fixed(const Ctl &c, const DevParams &P, double dt, double *q1) {
  double q0[4 * NB], pm[NB];
#pragma unroll
  for (int i = 0; i < NB; i++) {
    q0[i] = c.x[i];
    q0[i + NB] = c.y[i];
    q0[i + 2 * NB] = c.vx[i];
    q0[i + 3 * NB] = c.vy[i];
    pm[i] = c.mass[i];
  }
  double r[4 * NB];
  fargo_rk5_step<NB>(q0, pm, r, NB, dt, c.feelothers, P.indirect_term);
#pragma unroll
  for (int i = 0; i < 4 * NB; i++) q1[i] = r[i];
}

FARGO_HD void fargo_advance_rk5(Ctl &c, const DevParams &P, double dt, double t) {
  const int nb = c.nb;
  double q0[4 * FARGO_MAXPL], q1[4 * FARGO_MAXPL], pm[FARGO_MAXPL];
  for (int i = 0; i < 4 * nb; i++) q0[i] = q1[i] = 0.0;
  if (!P.forced_circular && nb > 0) {
    if (nb == 1) {
      fargo_rk5_fixed<1>(c, P, dt, q1);
    } else if (nb == 2) {
      fargo_rk5_fixed<2>(c, P, dt, q1);
    } else {
      for (int i = 0; i < nb; i++) {
        q0[i] = c.x[i];
        q0[i + nb] = c.y[i];
        q0[i + 2 * nb] = c.vx[i];
        q0[i + 3 * nb] = c.vy[i];
        pm[i] = c.mass[i];
      }
      fargo_rk5_step<0>(q0, pm, q1, nb, dt, c.feelothers, P.indirect_term);
    }
  }
  for (int i = 1 - (t >= P.releasedate); i < nb; i++) {
    if (!P.forced_circular) {
      c.x[i] = q1[i];
      c.y[i] = q1[i + nb];
      c.vx[i] = q1[i + 2 * nb];
      c.vy[i] = q1[i + 3 * nb];
    } else {
      double x = c.x[i], y = c.y[i];
      double theta = atan2(y, x);
      double vx = c.vx[i], vy = c.vy[i];
      double r = sqrt(x * x + y * y);
      double omega = (-y * vx + x * vy) / r / r;
      double dtheta = omega * dt;
      c.x[i] = r * cos(theta + dtheta);
      c.y[i] = r * sin(theta + dtheta);
      c.vx[i] = vx * cos(dtheta + theta) - vy * sin(dtheta + theta);
      c.vy[i] = vx * sin(dtheta + theta) + vy * cos(dtheta + theta);
    }
  }
  if (t < P.releasedate && nb > 0) {
    double x = c.x[0], y = c.y[0];
    double r = sqrt(x * x + y * y);
    double theta = atan2(y, x);
    double rdot = (P.releaseradius - r) / (P.releasedate - t);
    double omega = sqrt((1. + c.mass[0]) / r / r / r);
    double new_r = r + rdot * dt;
    double denom = r - new_r;
    double dtheta;
    if (denom != 0.0) dtheta = 2. * dt * r * omega / denom * (sqrt(r / new_r) - 1.);
    else dtheta = omega * dt;
    double vx = rdot;
    double vy = new_r * sqrt((1. + c.mass[0]) / new_r / new_r / new_r);
    c.x[0] = new_r * cos(dtheta + theta);
    c.y[0] = new_r * sin(dtheta + theta);
    c.vx[0] = vx * cos(dtheta + theta) - vy * sin(dtheta + theta);
    c.vy[0] = vx * sin(dtheta + theta) + vx * cos(dtheta + theta);
  }
}

// Planet parameters of a substep starting at time t: the smoothing of the disk's
// force on each FeelDisk body (AdvanceSystemFromDisk src/Pframeforce.cu:105-111;
// body 0 is the star, ComputeAccel(0,0,0) src/SourceEuler.cu:241) and the
// potential parameters of every planet (FillForcesArrays src/Pframeforce.cu:68-77).
FARGO_HD void fargo_planet_params(Ctl &c, const DevParams &P, double t) {
  const double t0 = c.PhysicalTimeInitial;
  const double taper = fargo_mass_taper(P, t);
  int nbody = 1;
  c.bx[0] = c.by[0] = c.brs2[0] = 0.0;
  for (int k = 0; k < c.nb; k++) {
    const double x = c.x[k], y = c.y[k], m = c.mass[k];
    // the distance to the star, and the thickness smoothing at it, serve both uses
    const double r = sqrt(x * x + y * y);
    const double smt = P.roche_smoothing ? 0.0 : fargo_smoothing(P, r, t, t0);
    if (c.feeldisk[k]) {
      const double sm = P.roche_smoothing ? r * pow(m / 3., 1. / 3.) * P.rochesmoothing : smt;
      c.bx[nbody] = x;
      c.by[nbody] = y;
      c.brs2[nbody] = sm * sm;
      nbody++;
    }
    const double mp = m * taper;
    const double PD = r;
    const double sm = P.roche_smoothing ? PD * pow((1.0 / 3.0 * mp), 1.0 / 3.0) * P.rochesmoothing : smt;
    c.px[k] = x;
    c.py[k] = y;
    c.pm[k] = mp;
    c.ps2[k] = sm * sm;
    c.pinvd3[k] = 1.0 / (PD * PD * PD);  // one divide (the reference divides three times)
  }
  c.nbody = nbody;
}

// Squared Keplerian speed of ApplySubKeplerianBoundary (src/SideEuler.cu:296-320)
// at ring radius r, before the self-gravity term.
FARGO_HD double fargo_vkep2(const DevParams &P, double r, double t, double t0) {
  const double f = 1.0 + P.sigmaslope - 2.0 * P.flaringindex;
  return 1.0 * 1.0 / r * (1.0 - f * fargo_pow(fargo_aspect_ratio(P, r, t, t0), 2.0) * fargo_pow(r, 2.0 * P.flaringindex));
}

// The Keplerian speed itself, before the frame term; csmean is the ring's mean
// sound speed, which the self-gravity form subtracts (Make1Dprofile(1)).
FARGO_HD double fargo_vkep(const DevParams &P, double r, double t, double t0, double csmean) {
  double v2 = fargo_vkep2(P, r, t, t0);
  if (P.self_gravity) v2 -= r * csmean;
  return sqrt(v2);
}

// The planetary part of one substep of length dt that started at time t
// (src/SourceEuler.cu:236-261): disk kicks with the indirect term
// (AdvanceSystemFromDisk), RK5 (AdvanceSystemRK5), the corotating frame update
// and RotatePsys; then the parameters of the next substep.  The disk
// accelerations and the indirect term are those of this substep.
FARGO_HD void fargo_planets_substep(Ctl &c, const DevParams &P, double dt, double t) {
  // dt = 0 (a substep padding the DT loop, or one after a device error): nothing
  // moves and the frame keeps its rate (the forced-circular and release-date
  // updates re-derive positions from angles and would not reproduce them exactly)
  if (dt == 0.0) {
    c.domega = 0.0;
    c.f32[CTL_F_DOMEGA] = 0.0f;
    return;
  }
  if (P.corotating) fargo_psys_info(c, P, 1);
  int b = 1;
  for (int k = 0; k < c.nb; k++) {
    if (c.feeldisk[k]) {
      c.vx[k] += dt * c.accx[b];
      c.vy[k] += dt * c.accy[b];
      c.vx[k] += dt * c.ind_x;
      c.vy[k] += dt * c.ind_y;
      b++;
    }
  }
  fargo_advance_rk5(c, P, dt, t);
  c.domega = 0.0;
  if (P.corotating && dt > 0.0) {
    const double OmegaNew = fargo_psys_info(c, P, 0) / dt;
    c.domega = OmegaNew - c.OmegaFrame;
    c.OmegaFrame = OmegaNew;
  }
  fargo_rotate_psys(c, c.OmegaFrame * dt);
  fargo_planet_params(c, P, t + dt);
  c.f32[CTL_F_OMEGA] = (float)c.OmegaFrame;
  c.f32[CTL_F_DOMEGA] = (float)c.domega;
}
