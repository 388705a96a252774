// setup.cpp -- host-side set-up of one disk: mesh, initial profiles, planets.
//
// Restates the initialisation sequence of main() (src/Main.cu:233-305): the
// 1D mesh (FillPolar1DArrays, src/SourceEuler.cu:66-162), the initial surface
// density and energy (src/Theo.cu, src/Pframeforce.cu:31-52), the planetary
// system (src/Psys.cu:168-217), the self-gravity kernel table (src/SgMain.cu:49-81)
// and InitEuler / InitGasVelocities (src/SourceEuler.cu:166-195,
// src/Pframeforce.cu:189-270).  Everything here runs once, in FP64, on the host;
// the per-step work is in the CUDA translation units.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "fargo_internal.h"

#define PI FARGO_PI

long fargo_nearest_pow2(long n) {  // NearestPowerOf2 src/Kernels.cu:346-355
  if (!n) return n;
  long x = 1;
  while (x < n) x <<= 1;
  return x;
}

DevParams host_dev_params(const fargo_params &p, int nb) {
  DevParams d;
  std::memset(&d, 0, sizeof(d));
  d.nrad = p.nrad;
  d.nsec = p.nsec;
  d.nb = nb;
  d.nsec2pot = (int)fargo_nearest_pow2(p.nsec);
  d.adiabatic = p.adiabatic;
  d.cooling = p.cooling;
  d.self_gravity = p.self_gravity;
  d.fast_transport = p.fast_transport;
  d.open_inner = p.open_inner;
  d.non_reflecting = p.non_reflecting;
  d.evanescent = p.evanescent;
  d.corotating = p.corotating;
  d.guiding_center = p.guiding_center;
  d.indirect_term = p.indirect_term;
  d.exclude_hill = p.exclude_hill;
  d.viscosity_alpha = p.viscosity_alpha;
  d.roche_smoothing = p.roche_smoothing;
  d.forced_circular = p.forced_circular;
  d.sloppy_cfl = p.sloppy_cfl;
  d.is_disk = p.is_disk;
  d.nu_dynamic = p.lambdadoubling != 0.0;
  d.DT = p.dt;
  d.aspectratio = p.aspectratio;
  d.flaringindex = p.flaringindex;
  d.sigmaslope = p.sigmaslope;
  d.sigma0 = p.sigma0;
  d.imposeddiskdrift = p.imposeddiskdrift;
  d.adiabaticindex = p.adiabaticindex;
  d.coolingtime0 = p.coolingtime0;
  d.thicknesssmoothing = p.thicknesssmoothing;
  d.rochesmoothing = p.rochesmoothing;
  d.masstaper = p.masstaper;
  d.releaseradius = p.releaseradius;
  d.releasedate = p.releasedate;
  d.transitionradius = p.transitionradius;
  d.transitionratio = p.transitionratio;
  d.transitionwidth = p.transitionwidth;
  d.lambdadoubling = p.lambdadoubling;
  d.viscosity = p.viscosity;
  d.alphaviscosity = p.alphaviscosity;
  d.cavityradius = p.cavityradius;
  d.cavityratio = p.cavityratio;
  d.cavitywidth = p.cavitywidth;
  return d;
}

// FillPolar1DArrays src/SourceEuler.cu:66-162 (radii.dat is not read).  Entries the
// reference leaves unset (index nrad of Rmed, Rsup, Surf, ... and invdiffRmed[0])
// are zero.
void host_fill_mesh(const fargo_params &p, HostState &h) {
  const int NRAD = p.nrad, NSEC = p.nsec;
  h.nrad = NRAD;
  h.nsec = NSEC;
  h.size_grid = (size_t)(NRAD + 1) * NSEC;
  for (auto *v : {&h.Radii, &h.Rinf, &h.Rmed, &h.Rsup, &h.Surf, &h.invRinf, &h.invSurf, &h.invRmed,
                  &h.invdiffRsup, &h.invdiffRmed})
    v->assign(NRAD + 1, 0.0);
  double drrsep = (p.rmax - p.rmin) / (double)NRAD;
  for (int i = 0; i <= NRAD; i++) {
    if (p.log_grid)
      h.Radii[i] = (double)p.rmin * exp((double)i / (double)NRAD * log((double)p.rmax / (double)p.rmin));
    else
      h.Radii[i] = p.rmin + drrsep * (double)i;
  }
  const std::vector<double> &R = h.Radii;
  for (int i = 0; i < NRAD; i++) {
    h.Rinf[i] = R[i];
    h.Rsup[i] = R[i + 1];
    double rm = 2.0 / 3.0 * (R[i + 1] * R[i + 1] * R[i + 1] - R[i] * R[i] * R[i]);
    rm = rm / (R[i + 1] * R[i + 1] - R[i] * R[i]);
    h.Rmed[i] = rm;
    h.Surf[i] = PI * (R[i + 1] * R[i + 1] - R[i] * R[i]) / (double)NSEC;
    h.invRmed[i] = 1.0 / rm;
    h.invSurf[i] = 1.0 / h.Surf[i];
    h.invdiffRsup[i] = 1.0 / (R[i + 1] - R[i]);
    h.invRinf[i] = 1.0 / R[i];
  }
  h.Rinf[NRAD] = R[NRAD];
  for (int i = 1; i < NRAD; i++) h.invdiffRmed[i] = 1.0 / (h.Rmed[i] - h.Rmed[i - 1]);
  // angle tables: InitComputeAccelKernel (src/Kernels.cu:161-162) and
  // FillForcesArraysKernel (src/Kernels.cu:1236-1238) evaluate the angle differently
  h.cosF.resize(NSEC);
  h.sinF.resize(NSEC);
  h.cosP.resize(NSEC);
  h.sinP.resize(NSEC);
  for (int j = 0; j < NSEC; j++) {
    h.cosF[j] = cos((2.0 * PI * (double)j) / (double)NSEC);
    h.sinF[j] = sin((2.0 * PI * (double)j) / (double)NSEC);
    double angle = (double)j / (double)NSEC * 2.0 * PI;
    h.cosP[j] = cos(angle);
    h.sinP[j] = sin(angle);
  }
}

static uint64_t splitmix64(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// Sigma / FillSigma / InitGasDensity, Energy / FillEnergy / InitGasEnergy
// (src/Theo.cu:13-52, src/Pframeforce.cu:31-52) + the seeded noise extension.
void host_init_density_energy(const fargo_params &p, HostState &h) {
  const int NRAD = p.nrad, NSEC = p.nsec;
  h.SigmaMed.assign(NRAD + 1, 0.0);
  h.SigmaInf.assign(NRAD + 1, 0.0);
  h.EnergyMed.assign(NRAD + 1, 0.0);
  h.Dens.assign(h.size_grid, 0.0);
  h.Energy.assign(h.size_grid, 0.0);
  auto sigma = [&](double r) {
    double cavity = 1.0;
    if (r < p.cavityradius) cavity = 1.0 / p.cavityratio;
    return cavity * p.scaling_factor * p.sigma0 * pow(r, -p.sigmaslope);
  };
  for (int i = 0; i < NRAD; i++) {
    h.SigmaMed[i] = sigma(h.Rmed[i]);
    h.SigmaInf[i] = sigma(h.Rinf[i]);
  }
  for (int i = 0; i < NRAD; i++)
    for (int j = 0; j < NSEC; j++) h.Dens[j + (size_t)i * NSEC] = h.SigmaMed[i];
  uint64_t seed = p.noise_seed;
  if (p.sigma_noise != 0.0)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        double u = (double)(splitmix64(seed) >> 11) * (1.0 / 9007199254740992.0);
        h.Dens[j + (size_t)i * NSEC] *= 1.0 + p.sigma_noise * (2.0 * u - 1.0);
      }
  if (p.adiabatic) {
    for (int i = 0; i < NRAD; i++)
      h.EnergyMed[i] = 1.0 / 1.0 / (p.adiabaticindex - 1.0) * p.sigma0 * pow(p.aspectratio, 2.0) *
                       pow(h.Rmed[i], -p.sigmaslope - 1.0 + 2.0 * p.flaringindex);
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) h.Energy[(size_t)i * NSEC + j] = h.EnergyMed[i];
    if (p.energy_noise != 0.0)
      for (int i = 0; i < NRAD; i++)
        for (int j = 0; j < NSEC; j++) {
          double u = (double)(splitmix64(seed) >> 11) * (1.0 / 9007199254740992.0);
          h.Energy[j + (size_t)i * NSEC] *= 1.0 + p.energy_noise * (2.0 * u - 1.0);
        }
  }
}

// InitPlanetarySystem tail (src/Psys.cu:187-211): CICPlanet moves each body to the
// interface above its ring; bodies were parsed by fargo_planets_read.
void host_init_planets(const fargo_params &p, const HostState &h, const fargo_planet *pl, int nb, Ctl &c) {
  c.nb = nb;
  for (int k = 0; k < nb; k++) {
    c.x[k] = pl[k].x;
    c.y[k] = pl[k].y;
    c.vx[k] = pl[k].vx;
    c.vy[k] = pl[k].vy;
    c.mass[k] = pl[k].mass;
    c.acc[k] = pl[k].acc;
    c.feeldisk[k] = pl[k].feel_disk;
    c.feelothers[k] = pl[k].feel_others;
    if (p.cic_planet) {
      double dist = c.x[k] / (1.0 + p.eccentricity);
      int j = 0;
      while (h.Rmed[j] < dist) j++;
      dist = h.Radii[j + 1];
      double mass = c.mass[k];
      c.x[k] = (double)dist * (1.0 + p.eccentricity);
      c.y[k] = 0.0;
      c.vy[k] = sqrt(1.0 * (1.0 + mass) / dist) * sqrt((1.0 - p.eccentricity) / (1.0 + p.eccentricity));
      c.vx[k] = -0.0000000001 * c.vy[k];
    }
  }
}

// compute_kernel src/SgMain.cu:49-81 (host, with the reference's single-precision coshf)
void host_sg_kernel(const fargo_params &p, HostState &h, DevParams &dp) {
  const int NRAD = p.nrad, NSEC = p.nsec;
  dp.sgp_eps = p.thicknesssmoothing * p.aspectratio;
  dp.sgp_rstep = log(h.Radii[NRAD] / h.Radii[0]) / (double)NRAD;
  dp.sgp_tstep = 2.0 * PI / (double)NSEC;
  const double eps = dp.sgp_eps;
  h.Kr.assign((size_t)2 * NRAD * NSEC, 0.0);
  h.Kt.assign((size_t)2 * NRAD * NSEC, 0.0);
  for (int i = 0; i < 2 * NRAD; i++) {
    double u;
    if (i < NRAD) u = log(h.Radii[i] / h.Radii[0]);
    else u = -log(h.Radii[2 * NRAD - i] / h.Radii[0]);
    for (int j = 0; j < NSEC; j++) {
      double theta = 2.0 * PI * (double)j / (double)NSEC;
      double Kr = 1.0 + eps * eps - cos(theta) * exp(-u);
      double base = eps * eps * exp(u) + 2.0 * (coshf(u) - cos(theta));
      Kr *= pow(base, -1.5);
      double Kt = sin(theta);
      Kt *= pow(base, -1.5);
      h.Kr[(size_t)i * NSEC + j] = Kr;
      h.Kt[(size_t)i * NSEC + j] = Kt;
    }
  }
}

// Init_planetarysys_withSG src/SgMain.cu:166-194.  The reference aborts at this
// point (Make1Dprofile(1) copies from SoundSpeed_d before it is allocated); the
// azimuthal mean of the radial self-gravity acceleration is used instead, as the
// function's comment intends.
void host_init_planets_sg(const fargo_params &p, const HostState &h, const std::vector<double> &axi, Ctl &c) {
  const int NRAD = p.nrad;
  for (int k = 0; k < c.nb; k++) {
    double r = c.x[k];
    double dist = (double)(r / (1. + p.eccentricity));
    int ipl = 0;
    while (ipl < NRAD - 2 && h.Rmed[ipl] <= dist) ipl++;
    double ri = h.Rmed[ipl], rip1 = h.Rmed[ipl + 1];
    double dr = rip1 - ri;
    double sgacc = (dist - ri) * axi[ipl + 1] + (rip1 - dist) * axi[ipl];
    sgacc /= dr;
    c.vy[k] *= (double)sqrt(1. - dist * dist * sgacc);
  }
}

// Make1Dprofile(1) src/Kernels.cu:610-645: ring means of SoundSpeed, summed in order
static void ring_mean_cs(const HostState &h, std::vector<double> &out) {
  out.assign(h.nrad + 1, 0.0);
  for (int i = 0; i < h.nrad; i++) {
    double sum = 0.0;
    for (int j = 0; j < h.nsec; j++) sum += h.SoundSpeed[(size_t)i * h.nsec + j];
    out[i] = sum / (double)h.nsec;
  }
}

// InitEuler (src/SourceEuler.cu:166-195): sound speed, pressure, temperature,
// then InitGasVelocities / InitVelocities (src/Pframeforce.cu:189-270).
void host_init_euler(const fargo_params &p, HostState &h, const DevParams &dp, Ctl &c) {
  const int NRAD = p.nrad, NSEC = p.nsec;
  const double t = 0.0;
  h.OmegaFrame = p.omegaframe;
  if (p.corotating) h.OmegaFrame = fargo_psys_info(c, dp, 2);
  c.OmegaFrame = h.OmegaFrame;
  h.SoundSpeed.assign(h.size_grid, 0.0);
  h.Pressure.assign(h.size_grid, 0.0);
  h.Temperature.assign(h.size_grid, 0.0);
  h.Vrad.assign(h.size_grid, 0.0);
  h.Vtheta.assign(h.size_grid, 0.0);
  // ComputeSoundSpeedKernel src/Kernels.cu:167-184
  for (int i = 0; i < NRAD; i++) {
    double AR = fargo_aspect_ratio(dp, h.Rmed[i], t, t);
    for (int j = 0; j < NSEC; j++) {
      size_t q = (size_t)i * NSEC + j;
      if (!p.adiabatic) h.SoundSpeed[q] = AR * sqrt(1.0 * 1.0 / h.Rmed[i]) * pow(h.Rmed[i], p.flaringindex);
      else h.SoundSpeed[q] = sqrt(p.adiabaticindex * (p.adiabaticindex - 1.0) * h.Energy[q] / h.Dens[q]);
    }
  }
  // ComputePressureFieldKernel / ComputeTemperatureFieldKernel src/Kernels.cu:187-213
  for (size_t q = 0; q < (size_t)NRAD * NSEC; q++) {
    if (!p.adiabatic) h.Pressure[q] = h.Dens[q] * h.SoundSpeed[q] * h.SoundSpeed[q];
    else h.Pressure[q] = (p.adiabaticindex - 1.0) * h.Energy[q];
    if (!p.adiabatic) h.Temperature[q] = 1.0 / 1.0 * h.Pressure[q] / h.Dens[q];
    else h.Temperature[q] = 1.0 / 1.0 * (p.adiabaticindex - 1.0) * h.Energy[q] / h.Dens[q];
  }
  ring_mean_cs(h, h.cs_mean);
  // Init_azimutalvelocity_withSG src/SourceEuler.cu:441-450 (Make1Dprofile(1) = mean cs)
  if (!p.centrifugal_balance && p.self_gravity) {
    for (int i = 0; i < NRAD; i++) {
      double invr = 1. / h.Rmed[i];
      double omegakep = sqrt(1.0 * 1.0 * invr * invr * invr);
      double omega = sqrt(omegakep * omegakep *
                              (1.0 - (1. + p.sigmaslope - 2.0 * p.flaringindex) * pow(p.aspectratio, 2.0) *
                                         pow(h.Rmed[i], 2.0 * p.flaringindex)) -
                          invr * h.cs_mean[i]);
      for (int j = 0; j < NSEC; j++) h.Vtheta[(size_t)i * NSEC + j] = h.Rmed[i] * omega;
    }
  }
  // cooling profiles (FillCoolingTime / FillQplus, src/Theo.cu:256-279)
  h.CoolingTimeMed.assign(NRAD + 1, 0.0);
  h.QplusMed.assign(NRAD + 1, 0.0);
  if (p.cooling) {
    for (int i = 0; i < NRAD; i++) h.CoolingTimeMed[i] = p.coolingtime0 * pow(h.Rmed[i], 2.0 + 2.0 * p.flaringindex);
    for (int i = 0; i < NRAD; i++) {
      double viscosity = fargo_fviscosity(dp, h.Rmed[i], h.cs_mean[i], t, t);
      h.QplusMed[i] = 2.25 * viscosity * p.sigma0 * pow(h.Rmed[i], -p.sigmaslope - 3.0);
    }
  }
  // InitVelocities src/Pframeforce.cu:256-270
  h.nu.assign(NRAD + 1, 0.0);
  for (int i = 0; i < NRAD; i++) h.nu[i] = fargo_fviscosity(dp, h.Rmed[i], h.cs_mean[i], t, t);
  h.nu[NRAD] = fargo_fviscosity(dp, h.Rmed[NRAD - 1], h.cs_mean[NRAD - 1], t, t);
  // InitGasVelocitiesKernel src/Kernels.cu:648-689
  for (int i = 0; i <= NRAD; i++) {
    double omega, r, ri;
    if (i == NRAD) { r = h.Rmed[NRAD - 1]; ri = h.Rinf[NRAD - 1]; }
    else { r = h.Rmed[i]; ri = h.Rinf[i]; }
    for (int j = 0; j < NSEC; j++) {
      size_t q = (size_t)i * NSEC + j;
      if (!p.self_gravity) {
        omega = sqrt(1.0 * 1.0 / r / r / r);
        h.Vtheta[q] = omega * r *
                      sqrt(1.0 - pow(p.aspectratio, 2.0) * pow(r, 2.0 * p.flaringindex) *
                                     (1. + p.sigmaslope - 2.0 * p.flaringindex));
      }
      h.Vtheta[q] -= h.OmegaFrame * r;
      if (i == NRAD) h.Vrad[q] = 0.0;
      else {
        h.Vrad[q] = p.imposeddiskdrift * p.sigma0 / h.SigmaInf[i] / ri;
        // the kernel's alpha branch (src/Kernels.cu:681) is unreachable: its int
        // flag receives `extern double ViscosityAlpha` (src/Pframeforce.cu:21), a
        // tiny double made of the int flag's bits, which converts to 0
        h.Vrad[q] -= 3.0 * h.nu[i] / r * (-p.sigmaslope + .5);
      }
    }
  }
  for (int j = 0; j < NSEC; j++) h.Vrad[j] = h.Vrad[(size_t)NRAD * NSEC + j] = 0.0;
}

// Per-ring constant table (rows of RingTab), FP64, evaluated with the same
// expressions the reference kernels evaluate per thread.
void host_ring_table(const fargo_params &p, const HostState &h, const DevParams &dp, std::vector<double> &tab) {
  const int n1 = p.nrad + 1, NSEC = p.nsec;
  tab.assign((size_t)RT_COUNT * n1, 0.0);
  // ring-major: the rows of one ring are adjacent (one base address per ring on the device)
  auto T = [&](int row, int i) -> double & { return tab[(size_t)i * RT_COUNT + row]; };
  auto at = [](const std::vector<double> &v, size_t i) { return i < v.size() ? v[i] : 0.0; };
  for (int i = 0; i < n1; i++) {
    T(RT_RINF, i) = h.Rinf[i];
    T(RT_RMED, i) = h.Rmed[i];
    T(RT_RSUP, i) = h.Rsup[i];
    T(RT_SURF, i) = h.Surf[i];
    T(RT_INVRINF, i) = h.invRinf[i];
    T(RT_INVSURF, i) = h.invSurf[i];
    T(RT_INVRMED, i) = h.invRmed[i];
    T(RT_INVDIFFRSUP, i) = h.invdiffRsup[i];
    T(RT_INVDIFFRMED, i) = h.invdiffRmed[i];
    double dxtheta = 2.0 * PI / (double)NSEC * h.Rmed[i];
    T(RT_DXTHETA, i) = dxtheta;
    T(RT_INVDXTHETA, i) = (i < p.nrad) ? 1.0 / dxtheta : 0.0;
    T(RT_DXTHETA_CFL, i) = h.Rmed[i] * 2.0 * PI / (double)NSEC;
    T(RT_SUPPTORQUE, i) = (i < p.nrad) ? p.imposeddiskdrift * 0.5 * pow(h.Rmed[i], -2.5 + p.sigmaslope) : 0.0;
    T(RT_CS, i) = (i < p.nrad && !p.adiabatic) ? at(h.SoundSpeed, (size_t)i * NSEC) : 0.0;
    T(RT_NU, i) = at(h.nu, i);
    T(RT_DRAD, i) = h.Rsup[i] - h.Rinf[i];
    if (i < p.nrad) {
      const double dxr = h.Rsup[i] - h.Rinf[i], dxt = h.Rmed[i] * 2.0 * PI / (double)NSEC;
      T(RT_INVDRAD, i) = 1.0 / dxr;
      T(RT_INVDXTHETA_CFL, i) = 1.0 / dxt;
      T(RT_INVMIND, i) = 1.0 / ((dxt < dxr) ? dxt : dxr);
    }
    // time-independent parts of the edge speed and of the viscosity profile (the
    // device evaluates them in full when the aspect ratio changes in time)
    T(RT_VKEP2, i) = fargo_vkep2(dp, h.Rmed[i], 0.0, 0.0);
    T(RT_R15, i) = pow(h.Rmed[i], 1.5);
    T(RT_CAVFAC, i) = fargo_cavity_factor(dp, h.Rmed[i], 0.0, 0.0);
    T(RT_AZSHIFT, i) = (i < p.nrad) ? h.invRmed[i] * (double)NSEC / 2.0 / PI : 0.0;
    T(RT_SIGMAMED, i) = at(h.SigmaMed, i);
    T(RT_INVSIGMAMED, i) = at(h.SigmaMed, i) != 0.0 ? 1.0 / at(h.SigmaMed, i) : 0.0;
    T(RT_ENERGYMED, i) = at(h.EnergyMed, i);
    T(RT_COOLTIME, i) = at(h.CoolingTimeMed, i);
    T(RT_QPLUSMED, i) = at(h.QplusMed, i);
    T(RT_SGSQRT, i) = (i < p.nrad) ? sqrt(h.Rmed[i] / h.Rmed[0]) : 0.0;
    T(RT_SGRATIO, i) = (i < p.nrad) ? h.Rmed[i] / h.Rmed[0] : 0.0;
    T(RT_CSMEAN, i) = at(h.cs_mean, i);
    if (p.self_gravity && i < p.nrad) {
      double divRmed = h.Rmed[i] / h.Rmed[0];
      double normaccr = dp.sgp_rstep * dp.sgp_tstep / ((double)(2 * p.nrad) * (double)NSEC);
      double normacct = normaccr;
      normaccr /= sqrt(divRmed);
      normacct /= (divRmed * sqrt(divRmed));
      T(RT_SGNORMR, i) = normaccr;
      T(RT_SGNORMT, i) = normacct;
    }
  }
}
