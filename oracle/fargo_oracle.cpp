/*
 * fargo_oracle.cpp -- TEST INFRASTRUCTURE, NOT THE PRODUCT.
 *
 * FP64 CPU restatement of the reference FARGO-ADSG hydro step of
 * MatiasFloresS/CudaProtoplanetaryDisks.  It is the checker for the CUDA path
 * (tests/, __graft_entry__.smoke()) and the timed CPU baseline (bench.py's
 * cpu_baseline / --impl reference), nothing else: no product code path may call
 * it.  The reference has no CPU implementation of these substeps (every substep
 * is a CUDA kernel in src/Kernels.cu); each function below restates one reference
 * kernel or host driver, cites it, and keeps its arithmetic in the same order so
 * that, compiled with -ffp-contract=off, it reproduces the reference sources
 * compiled for the CPU bit for bit (oracle/ref_emul, tests/test_oracle_pin.py).
 *
 * Kernel-launch semantics are kept: one loop nest per reference launch, so every
 * loop reads the values that existed before it (reference launches are separated
 * by cudaDeviceSynchronize).  Loops over rings run under OpenMP; every sum whose
 * order matters is done sequentially inside one ring or in the reference's
 * DeviceReduce order (src/Kernels.cu:253-394), so results do not depend on the
 * thread count.
 */
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../include/fargo_gb300.h"
#include "fft_ref.h"

#ifdef _OPENMP
#include <omp.h>
#endif

/* include/Fondam.cuh */
#define G 1.0
#define PI 3.14159265358979323844
#define MU 1.0
#define R 1.0
#define CFLSECURITY 0.5
#define CVNR 1.41
#define YES 1
#define NO 0

namespace {

typedef std::vector<double> vec;

static long nearest_pow2(long n) { /* NearestPowerOf2 src/Kernels.cu:346-355 */
  if (!n) return n;
  int x = 1;
  while (x < n) x <<= 1;
  return x;
}

/* DeviceReduce src/Kernels.cu:364-394 with DeviceReduceKernel<false> 253-343:
   32-thread blocks, blocks = min(ceil(pow2(N)/32), 1024); per-thread strided pair
   sums, pairwise tree inside the block, sequential host sum of block partials.
   IsPow2 (src/Kernels.cu:358-361) is false for every N > 1. */
static double device_reduce(const double *in, int N) {
  const int threads = 32;
  int blocks = std::min((int)((nearest_pow2(N) + threads - 1) / threads), 1024);
  bool is_pow2 = (N == 1);
  unsigned gridSize = (unsigned)threads * 2u * (unsigned)blocks;
  std::vector<double> part(blocks);
  for (int b = 0; b < blocks; ++b) {
    double s[32];
    for (int t = 0; t < threads; ++t) {
      unsigned i = (unsigned)b * threads * 2u + (unsigned)t;
      double mySum = 0.0;
      while (i < (unsigned)N) {
        mySum += in[i];
        /* for N == 1 (IsPow2 true) the reference reads in[32], past the array;
           that element counts as zero here */
        if ((is_pow2 || i + threads < (unsigned)N) && i + threads < (unsigned)N) mySum += in[i + threads];
        i += gridSize;
      }
      s[t] = mySum;
    }
    for (int off = 16; off > 0; off >>= 1)
      for (int t = 0; t < off; ++t) s[t] = s[t] + s[t + off];
    part[b] = s[0];
  }
  double sum = 0.0;
  for (int b = 0; b < blocks; ++b) sum += part[b];
  return sum;
}

static double max2(double a, double b) { return (b > a) ? b : a; } /* src/Kernels.cu:1363 */
static double min2(double a, double b) { return (b < a) ? b : a; } /* src/Kernels.cu:1370 */

struct Psys {
  int nb = 0;
  vec x, y, vx, vy, mass, acc;
  std::vector<int> feeldisk, feelothers;
};

struct Oracle {
  fargo_params P;
  int NRAD, NSEC, size_grid, nsec2pot;
  /* 1D mesh (FillPolar1DArrays) */
  vec Radii, Rinf, Rmed, Rsup, Surf, invRinf, invSurf, invRmed, invdiffRsup, invdiffRmed, powRmed;
  vec SigmaMed, SigmaInf, EnergyMed, CoolingTimeMed, QplusMed, viscosity_array, GLOBAL_bufarray;
  vec GLOBAL_AxiSGAccr;
  /* 2D fields */
  vec Dens, Vrad, Vtheta, Energy, SoundSpeed, Pressure, Temperature, Potential;
  vec VradInt, VthetaInt, VradNew, VthetaNew, EnergyInt, EnergyNew, DensInt, TemperInt, Qplus;
  vec DivergenceVelocity, DRR, DPP, DRP, TAURR, TAURP, TAUPP;
  vec RadMomP, RadMomM, ThetaMomP, ThetaMomM, Work, QRStar, DensStar, dq, VthetaRes, TempShift;
  vec Vresidual, DT2D, DT1D, newDT, Vmoy, VMed, LostByDisk;
  std::vector<int> Nshift, NoSplitAdvection;
  vec CellAbscissa, CellOrdinate, fxo, fyo;
  /* self-gravity */
  vec Kr_aux, Kt_aux, SG_Accr, SG_Acct;
  std::vector<fftref::cplx> Kr_hat, Kt_hat;
  double SGP_eps = 0, SGP_rstep = 0, SGP_tstep = 0;
  /* scalars */
  double PhysicalTime = 0.0, PhysicalTimeInitial = 0.0, OmegaFrame = 0.0, MassTaper = 0.0;
  double LostMass = 0.0, last_dt = 0.0;
  long long substeps = 0;
  int last_cfl = 0;
  double IndirectTermX = 0.0, IndirectTermY = 0.0; /* static Pair IndirectTerm, Pframeforce.cu:24 */
  double DiskOnPrimaryX = 0.0, DiskOnPrimaryY = 0.0;
  double XplanetMark = 0.0, YplanetMark = 0.0;      /* Psys.cu:79 statics */
  Psys sys;
  std::string err;

  /* ------------------------------------------------------------------ */
  /* src/Viscosity.cu:93-107 AspectRatioHost (== AspectRatioDevice, Kernels.cu:1377) */
  double AspectRatio(double r) const {
    double aspectratio, rmin, rmax, scale;
    aspectratio = P.aspectratio;
    rmin = P.transitionradius - P.transitionwidth * P.aspectratio;
    rmax = P.transitionradius + P.transitionwidth * P.aspectratio;
    scale = 1.0 + (PhysicalTime - PhysicalTimeInitial) * P.lambdadoubling;
    rmin *= scale;
    rmax *= scale;
    if (r < rmin) aspectratio *= P.transitionratio;
    if ((r >= rmin) && (r <= rmax)) aspectratio *= exp((rmax - r) / (rmax - rmin) * log(P.transitionratio));
    return aspectratio;
  }
  /* src/Viscosity.cu:33-50 FViscosity */
  double FViscosity(double r) const {
    double viscosity, rmin, rmax, scale;
    int i = 0;
    viscosity = P.viscosity;
    if (P.viscosity_alpha) {
      while (Rmed[i] < r) i++;
      viscosity = P.alphaviscosity * GLOBAL_bufarray[i] * GLOBAL_bufarray[i] * pow(r, 1.5);
    }
    rmin = P.cavityradius - P.cavitywidth * P.aspectratio;
    rmax = P.cavityradius + P.cavitywidth * P.aspectratio;
    scale = 1.0 + (PhysicalTime - PhysicalTimeInitial) * P.lambdadoubling;
    rmin *= scale;
    rmax *= scale;
    if (r < rmin) viscosity *= P.cavityratio;
    if ((r >= rmin) && (r <= rmax)) viscosity *= exp((rmax - r) / (rmax - rmin) * log(P.cavityratio));
    return viscosity;
  }
  /* src/Force.cu:137-142 */
  double Compute_smoothing(double r) const {
    return P.thicknesssmoothing * AspectRatio(r) * pow(r, 1.0 + P.flaringindex);
  }
  /* src/Theo.cu:13-21 */
  double Sigma(double r) const {
    double cavity = 1.0;
    if (r < P.cavityradius) cavity = 1.0 / P.cavityratio;
    return cavity * P.scaling_factor * P.sigma0 * pow(r, -P.sigmaslope);
  }
  /* src/Theo.cu:37-49 */
  double EnergyProfile(double r) const {
    return R / MU / (P.adiabaticindex - 1.0) * P.sigma0 * pow(P.aspectratio, 2.0) *
           pow(r, -P.sigmaslope - 1.0 + 2.0 * P.flaringindex);
  }

  /* ------------------------------------------------------------------ */
  /* FillPolar1DArrays src/SourceEuler.cu:66-162 (no radii.dat path). */
  void FillPolar1DArrays() {
    int n1 = NRAD + 1;
    for (vec *v : {&Radii, &Rinf, &Rmed, &Rsup, &Surf, &invRinf, &invSurf, &invRmed, &invdiffRsup,
                   &invdiffRmed, &powRmed})
      v->assign(n1, 0.0);
    double drrsep = (P.rmax - P.rmin) / (double)NRAD;
    for (int i = 0; i <= NRAD; i++) {
      if (P.log_grid)
        Radii[i] = (double)P.rmin * exp((double)i / (double)NRAD * log((double)P.rmax / (double)P.rmin));
      else
        Radii[i] = P.rmin + drrsep * (double)i;
    }
    for (int i = 0; i < NRAD; i++) {
      Rinf[i] = Radii[i];
      Rsup[i] = Radii[i + 1];
      double rm = 2.0 / 3.0 * (Radii[i + 1] * Radii[i + 1] * Radii[i + 1] - Radii[i] * Radii[i] * Radii[i]);
      rm = rm / (Radii[i + 1] * Radii[i + 1] - Radii[i] * Radii[i]);
      Rmed[i] = rm;
      Surf[i] = PI * (Radii[i + 1] * Radii[i + 1] - Radii[i] * Radii[i]) / (double)NSEC;
      invRmed[i] = 1.0 / rm;
      invSurf[i] = 1.0 / Surf[i];
      invdiffRsup[i] = 1.0 / (Radii[i + 1] - Radii[i]);
      invRinf[i] = 1.0 / Radii[i];
    }
    Rinf[NRAD] = Radii[NRAD];
    for (int i = 0; i < NRAD; i++) {
      if (i > 0) invdiffRmed[i] = 1.0 / (Rmed[i] - Rmed[i - 1]);
      powRmed[i] = pow(Rmed[i], -2.5 + P.sigmaslope);
    }
  }

  static uint64_t splitmix64(uint64_t &s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }

  /* Make1Dprofile(1) src/Kernels.cu:610-645: the option always averages SoundSpeed. */
  void Make1Dprofile_cs() {
    for (int i = 0; i < NRAD; i++) {
      double sum = 0.0;
      for (int j = 0; j < NSEC; j++) sum += SoundSpeed[(size_t)i * NSEC + j];
      GLOBAL_bufarray[i] = sum / (double)NSEC;
    }
  }

  /* ------------------------------------------------------------------ */
  bool init(const fargo_params *p, const fargo_planet *pl, int nb) {
    P = *p;
    NRAD = P.nrad;
    NSEC = P.nsec;
    if (NRAD < 4 || NSEC < 4) { err = "nrad and nsec must be >= 4"; return false; }
    size_grid = (NRAD + 1) * NSEC;
    nsec2pot = (int)nearest_pow2(NSEC);
    size_t sg = (size_t)size_grid;
    for (vec *v : {&Dens, &Vrad, &Vtheta, &Energy, &SoundSpeed, &Pressure, &Temperature, &Potential,
                   &VradInt, &VthetaInt, &VradNew, &VthetaNew, &EnergyInt, &EnergyNew, &DensInt,
                   &TemperInt, &Qplus, &DivergenceVelocity, &DRR, &DPP, &DRP, &TAURR, &TAURP, &TAUPP,
                   &RadMomP, &RadMomM, &ThetaMomP, &ThetaMomM, &Work, &QRStar, &DensStar, &dq,
                   &VthetaRes, &TempShift, &Vresidual, &CellAbscissa, &CellOrdinate})
      v->assign(sg, 0.0);
    DT2D.assign((size_t)NRAD * NSEC, 0.0);
    fxo.assign((size_t)NRAD * NSEC, 0.0);
    fyo.assign((size_t)NRAD * NSEC, 0.0);
    DT1D.assign(NRAD, 0.0);
    newDT.assign(NRAD, 0.0);
    Vmoy.assign(sg, 0.0);
    VMed.assign(NRAD, 0.0);
    LostByDisk.assign(NSEC, 0.0);
    Nshift.assign(NRAD, 0);
    NoSplitAdvection.assign(NRAD, 0);
    for (vec *v : {&SigmaMed, &SigmaInf, &EnergyMed, &CoolingTimeMed, &QplusMed, &viscosity_array,
                   &GLOBAL_bufarray, &GLOBAL_AxiSGAccr})
      v->assign(NRAD + 1, 0.0);

    /* main(): src/Main.cu:245-305 */
    FillPolar1DArrays();
    /* InitPlanetarySystem src/Psys.cu:168-217 (bodies already parsed by the caller;
       CICPlanet moves them to the next interface) */
    sys.nb = nb;
    sys.x.assign(nb + 1, 0.0); sys.y.assign(nb + 1, 0.0); sys.vx.assign(nb + 1, 0.0);
    sys.vy.assign(nb + 1, 0.0); sys.mass.assign(nb + 1, 0.0); sys.acc.assign(nb + 1, 0.0);
    sys.feeldisk.assign(nb + 1, 1); sys.feelothers.assign(nb + 1, 1);
    for (int k = 0; k < nb; k++) {
      sys.x[k] = pl[k].x; sys.y[k] = pl[k].y; sys.vx[k] = pl[k].vx; sys.vy[k] = pl[k].vy;
      sys.mass[k] = pl[k].mass; sys.acc[k] = pl[k].acc;
      sys.feeldisk[k] = pl[k].feel_disk; sys.feelothers[k] = pl[k].feel_others;
    }
    if (P.cic_planet) {
      for (int k = 0; k < nb; k++) {
        double dist = sys.x[k] / (1.0 + P.eccentricity);
        int j = 0;
        while (Rmed[j] < dist) j++;
        dist = Radii[j + 1];
        double mass = sys.mass[k];
        sys.x[k] = (double)dist * (1.0 + P.eccentricity);
        sys.y[k] = 0.0;
        sys.vy[k] = sqrt(G * (1.0 + mass) / dist) * sqrt((1.0 - P.eccentricity) / (1.0 + P.eccentricity));
        sys.vx[k] = -0.0000000001 * sys.vy[k];
      }
    }
    /* InitGasDensity src/Pframeforce.cu:31-40 -> FillSigma src/Theo.cu:25-32 */
    for (int i = 0; i < NRAD; i++) {
      SigmaMed[i] = Sigma(Rmed[i]);
      SigmaInf[i] = Sigma(Rinf[i]);
    }
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) Dens[j + (size_t)i * NSEC] = SigmaMed[i];
    uint64_t seed = P.noise_seed;
    if (P.sigma_noise != 0.0)
      for (int i = 0; i < NRAD; i++)
        for (int j = 0; j < NSEC; j++) {
          double u = (double)(splitmix64(seed) >> 11) * (1.0 / 9007199254740992.0);
          Dens[j + (size_t)i * NSEC] *= 1.0 + P.sigma_noise * (2.0 * u - 1.0);
        }
    /* InitGasEnergy src/Pframeforce.cu:44-52 -> FillEnergy src/Theo.cu:247-252 */
    if (P.adiabatic) {
      for (int i = 0; i < NRAD; i++) EnergyMed[i] = EnergyProfile(Rmed[i]);
      for (int i = 0; i < NRAD; i++)
        for (int j = 0; j < NSEC; j++) Energy[(size_t)i * NSEC + j] = EnergyMed[i];
      if (P.energy_noise != 0.0)
        for (int i = 0; i < NRAD; i++)
          for (int j = 0; j < NSEC; j++) {
            double u = (double)(splitmix64(seed) >> 11) * (1.0 / 9007199254740992.0);
            Energy[j + (size_t)i * NSEC] *= 1.0 + P.energy_noise * (2.0 * u - 1.0);
          }
    }
    /* self-gravity set-up src/Main.cu:268-290 */
    if (P.self_gravity) {
      SGP_eps = P.thicknesssmoothing * P.aspectratio;
      SGP_rstep = log(Radii[NRAD] / Radii[0]) / (double)NRAD;
      SGP_tstep = 2.0 * PI / (double)NSEC;
      compute_kernel();
      SG_Accr.assign(sg, 0.0);
      SG_Acct.assign(sg, 0.0);
      compute_selfgravity(0.0, false);
      Init_planetarysys_withSG();
    }
    OmegaFrame = P.omegaframe;
    if (P.corotating) OmegaFrame = GetPsysInfo(2 /* FREQUENCY */);
    /* Initialization -> InitEuler src/SourceEuler.cu:166-195 */
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        CellAbscissa[(size_t)i * NSEC + j] = Rmed[i] * cos((2.0 * PI * (double)j) / (double)NSEC);
        CellOrdinate[(size_t)i * NSEC + j] = Rmed[i] * sin((2.0 * PI * (double)j) / (double)NSEC);
      }
    ComputeSoundSpeed();
    ComputePressureField();
    ComputeTemperatureField();
    InitGasVelocities();
    PhysicalTimeInitial = PhysicalTime;
    return true;
  }

  /* InitGasVelocities src/Pframeforce.cu:189-253 (+ InitVelocities 256-270) */
  void InitGasVelocities() {
    /* CentrifugalBalance builds vt_cent, which the velocity kernel never reads
       (src/Kernels.cu:675 is commented out): no effect on the state. */
    if (!P.centrifugal_balance && P.self_gravity) {
      /* Init_azimutalvelocity_withSG src/SourceEuler.cu:441-450 */
      Make1Dprofile_cs();
      for (int i = 0; i < NRAD; i++) {
        double invr = 1. / Rmed[i];
        double omegakep = sqrt(G * 1.0 * invr * invr * invr);
        double omega = sqrt(omegakep * omegakep *
                                (1.0 - (1. + P.sigmaslope - 2.0 * P.flaringindex) * pow(P.aspectratio, 2.0) *
                                           pow(Rmed[i], 2.0 * P.flaringindex)) -
                            invr * GLOBAL_bufarray[i]);
        for (int j = 0; j < NSEC; j++) Vtheta[(size_t)i * NSEC + j] = Rmed[i] * omega;
      }
    }
    if (P.viscosity_alpha) Make1Dprofile_cs();
    if (P.cooling) {
      for (int i = 0; i < NRAD; i++) CoolingTimeMed[i] = P.coolingtime0 * pow(Rmed[i], 2.0 + 2.0 * P.flaringindex);
      for (int i = 0; i < NRAD; i++) {
        double viscosity = FViscosity(Rmed[i]);
        QplusMed[i] = 2.25 * viscosity * P.sigma0 * pow(Rmed[i], -P.sigmaslope - 3.0);
      }
    }
    for (int i = 0; i < NRAD; i++) viscosity_array[i] = FViscosity(Rmed[i]);
    viscosity_array[NRAD] = FViscosity(Rmed[NRAD - 1]);
    /* InitGasVelocitiesKernel src/Kernels.cu:648-689 */
    for (int i = 0; i <= NRAD; i++) {
      double omega, r, ri;
      if (i == NRAD) { r = Rmed[NRAD - 1]; ri = Rinf[NRAD - 1]; }
      else { r = Rmed[i]; ri = Rinf[i]; }
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        if (!P.self_gravity) {
          omega = sqrt(G * 1.0 / r / r / r);
          Vtheta[c] = omega * r *
                      sqrt(1.0 - pow(P.aspectratio, 2.0) * pow(r, 2.0 * P.flaringindex) *
                                     (1. + P.sigmaslope - 2.0 * P.flaringindex));
        }
        Vtheta[c] -= OmegaFrame * r;
        if (i == NRAD) Vrad[c] = 0.0;
        else {
          Vrad[c] = P.imposeddiskdrift * P.sigma0 / SigmaInf[i] / ri;
          /* The alpha branch of the kernel (src/Kernels.cu:681) is never taken: the
             caller passes `extern double ViscosityAlpha` (src/Pframeforce.cu:21),
             whose bits are the int flag and its neighbour, to the kernel's int
             parameter, and that tiny double converts to 0. */
          Vrad[c] -= 3.0 * viscosity_array[i] / r * (-P.sigmaslope + .5);
        }
      }
    }
    for (int j = 0; j < NSEC; j++) Vrad[j] = Vrad[(size_t)NRAD * NSEC + j] = 0.0;
  }

  /* ------------------------------------------------------------------ */
  /* ComputeSoundSpeedKernel src/Kernels.cu:167-184 */
  void ComputeSoundSpeed() {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++) {
      double AR = P.adiabatic ? 0.0 : AspectRatio(Rmed[i]);
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        if (!P.adiabatic) SoundSpeed[c] = AR * sqrt(G * 1.0 / Rmed[i]) * pow(Rmed[i], P.flaringindex);
        else SoundSpeed[c] = sqrt(P.adiabaticindex * (P.adiabaticindex - 1.0) * Energy[c] / Dens[c]);
      }
    }
  }
  /* ComputePressureFieldKernel src/Kernels.cu:187-200 */
  void ComputePressureField() {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        if (!P.adiabatic) Pressure[c] = Dens[c] * SoundSpeed[c] * SoundSpeed[c];
        else Pressure[c] = (P.adiabaticindex - 1.0) * Energy[c];
      }
  }
  /* ComputeTemperatureFieldKernel src/Kernels.cu:203-213 */
  void ComputeTemperatureField() {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        if (!P.adiabatic) Temperature[c] = MU / R * Pressure[c] / Dens[c];
        else Temperature[c] = MU / R * (P.adiabaticindex - 1.0) * Energy[c] / Dens[c];
      }
  }

  /* ------------------------------------------------------------------ */
  /* ConditionCFL src/SourceEuler.cu:520-546; kernels src/Kernels.cu:1267-1359 */
  int ConditionCFL(double DeltaT) {
    for (int i = 0; i < NRAD; i++) {
      Vmoy[i] = 0.0;
      for (int j = 0; j < NSEC; j++) Vmoy[i] += Vtheta[(size_t)i * NSEC + j];
      Vmoy[i] /= (double)NSEC;
    }
    std::fill(DT2D.begin(), DT2D.end(), 0.0);
    std::fill(DT1D.begin(), DT1D.end(), 0.0);
#pragma omp parallel for schedule(static)
    for (int i = 1; i < NRAD; i++) {
      double dxrad = Rsup[i] - Rinf[i];
      double dxtheta = Rmed[i] * 2.0 * PI / (double)NSEC;
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        if (P.fast_transport) Vresidual[c] = Vtheta[c] - Vmoy[i];
        else Vresidual[c] = Vtheta[c];
        double invdt1 = SoundSpeed[c] / (min2(dxrad, dxtheta));
        double invdt2 = fabs(Vrad[c]) / dxrad;
        double invdt3 = fabs(Vresidual[c]) / dxtheta;
        double dvr = Vrad[c + NSEC] - Vrad[c];
        double dvt = Vtheta[(size_t)i * NSEC + (j + 1) % NSEC] - Vtheta[c];
        if (dvr >= 0.0) dvr = 1e-10; else dvr = -dvr;
        if (dvt >= 0.0) dvt = 1e-10; else dvt = -dvt;
        double invdt4 = max2(dvr / dxrad, dvt / dxtheta);
        invdt4 *= 4.0 * CVNR * CVNR;
        double dt = CFLSECURITY / sqrt(invdt1 * invdt1 + invdt2 * invdt2 + invdt3 * invdt3 + invdt4 * invdt4);
        DT2D[c] = dt;
      }
    }
    for (int i = 0; i < NRAD; i++) {
      double newdt = 1e30;
      if (i > 0 && i < NRAD) {
        newDT[i] = newdt;
        for (int k = 0; k < NSEC; k++)
          if (DT2D[(size_t)i * NSEC + k] < newDT[i]) newDT[i] = DT2D[(size_t)i * NSEC + k];
      }
      if (i < NRAD - 1) {
        double dt = 2.0 * PI * CFLSECURITY / (double)NSEC / fabs(Vmoy[i] * invRmed[i] - Vmoy[i + 1] * invRmed[i + 1]);
        DT1D[i] = dt;
      }
    }
    double newdt = newDT[1];
    for (int i = 2; i < NRAD; i++)
      if (newDT[i] < newdt) newdt = newDT[i];
    for (int i = 0; i < NRAD - 1; i++)
      if (DT1D[i] < newdt) newdt = DT1D[i];
    if (DeltaT < newdt) newdt = DeltaT;
    return (int)(ceil(DeltaT / newdt));
  }

  /* ------------------------------------------------------------------ */
  /* ComputeForceKernel src/Kernels.cu:693-729 for level k = 0 (a = 0, rh = 0 at
     every call site, src/SideEuler.cu:245, so all dimfxy levels coincide and only
     the "outer" arrays are non-zero) + DeviceReduce (src/Force.cu:390-393). */
  void ComputeAccel(double x, double y, double rsmoothing, double *ax, double *ay) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        double cellmass = Surf[i] * Dens[c];
        double dx = CellAbscissa[c] - x;
        double dy = CellOrdinate[c] - y;
        double d2 = dx * dx + dy * dy;
        double dist2 = d2 + rsmoothing * rsmoothing;
        double distance = sqrt(dist2);
        double InvDist3 = 1.0 / dist2 / distance;
        double hill_cut = 1.;
        fxo[c] = G * cellmass * dx * InvDist3 * hill_cut;
        fyo[c] = G * cellmass * dy * InvDist3 * hill_cut;
      }
    double fx_inner = 0.0, fy_inner = 0.0;  /* DeviceReduce of the all-zero inner arrays */
    double fx_outer = device_reduce(fxo.data(), NRAD * NSEC);
    double fy_outer = device_reduce(fyo.data(), NRAD * NSEC);
    *ax = fx_inner + fx_outer;  /* ComputeAccel src/SideEuler.cu:242-255 */
    *ay = fy_inner + fy_outer;
  }

  /* FillForcesArrays src/Pframeforce.cu:56-94; kernel src/Kernels.cu:1226-1253 */
  void FillForcesArrays() {
    IndirectTermX = -DiskOnPrimaryX;
    IndirectTermY = -DiskOnPrimaryY;
    if (!P.indirect_term) { IndirectTermX = 0.0; IndirectTermY = 0.0; }
    std::fill(Potential.begin(), Potential.end(), 0.0);
    for (int k = 0; k < sys.nb; k++) {
      double xplanet = sys.x[k], yplanet = sys.y[k];
      double mplanet = sys.mass[k] * MassTaper;
      double PlanetDistance = sqrt(xplanet * xplanet + yplanet * yplanet);
      double InvPlanetDistance3 = 1.0 / PlanetDistance / PlanetDistance / PlanetDistance;
      double RRoche = PlanetDistance * pow((1.0 / 3.0 * mplanet), 1.0 / 3.0);
      double smoothing = P.roche_smoothing ? RRoche * P.rochesmoothing : Compute_smoothing(PlanetDistance);
      double smooth = smoothing * smoothing;
#pragma omp parallel for schedule(static)
      for (int i = 0; i < NRAD; i++) {
        double InvDistance = 1.0 / Rmed[i];
        for (int j = 0; j < NSEC; j++) {
          size_t c = (size_t)i * NSEC + j;
          double angle = (double)j / (double)NSEC * 2.0 * PI;
          double x = Rmed[i] * cos(angle);
          double y = Rmed[i] * sin(angle);
          double distance = (x - xplanet) * (x - xplanet) + (y - yplanet) * (y - yplanet);
          double distancesmooth = sqrt(distance + smooth);
          double pot = -G * mplanet / distancesmooth;
          if (P.indirect_term == YES) pot += G * mplanet * InvPlanetDistance3 * (x * xplanet + y * yplanet);
          Potential[c] += pot;
          if (k == 0) {
            pot = -G * 1.0 * InvDistance;
            pot -= IndirectTermX * x + IndirectTermY * y;
            Potential[c] += pot;
          }
        }
      }
    }
  }

  /* AdvanceSystemFromDisk src/Pframeforce.cu:97-121 */
  void AdvanceSystemFromDisk(double dt) {
    for (int k = 0; k < sys.nb; k++) {
      if (sys.feeldisk[k]) {
        double m = sys.mass[k], x = sys.x[k], y = sys.y[k];
        double r = sqrt(x * x + y * y);
        double smoothing = P.roche_smoothing ? r * pow(m / 3., 1. / 3.) * P.rochesmoothing : Compute_smoothing(r);
        double gx, gy;
        ComputeAccel(x, y, smoothing, &gx, &gy);
        sys.vx[k] += dt * gx;
        sys.vy[k] += dt * gy;
        sys.vx[k] += dt * IndirectTermX;
        sys.vy[k] += dt * IndirectTermY;
      }
    }
  }

  /* RungeKutta / DerivMotionRK5 / TranslatePlanetRK5 src/RungeKutta.cu:8-75 */
  void DerivMotionRK5(const double *q_init, const double *PlanetMasses, double *deriv, int nb, double dt,
                      const int *feelothers) {
    const double *x = q_init, *y = x + nb, *vx = y + nb, *vy = vx + nb;
    double *derivx = deriv, *derivy = derivx + nb, *derivvx = derivy + nb, *derivvy = derivvx + nb;
    std::vector<double> Dist(nb);
    for (int i = 0; i < nb; i++) Dist[i] = sqrt(x[i] * x[i] + y[i] * y[i]);
    for (int i = 0; i < nb; i++) {
      derivx[i] = vx[i];
      derivy[i] = vy[i];
      derivvx[i] = -G * 1.0 / Dist[i] / Dist[i] / Dist[i] * x[i];
      derivvy[i] = -G * 1.0 / Dist[i] / Dist[i] / Dist[i] * y[i];
      for (int j = 0; j < nb; j++) {
        if (P.indirect_term == YES) {
          derivvx[i] -= G * PlanetMasses[j] / Dist[j] / Dist[j] / Dist[j] * x[j];
          derivvy[i] -= G * PlanetMasses[j] / Dist[j] / Dist[j] / Dist[j] * y[j];
        }
        if ((j != i) && (feelothers[i] == YES)) {
          derivvx[i] += G * PlanetMasses[j] / Dist[j] / Dist[j] / Dist[j] * (x[j] - x[i]);
          derivvy[i] += G * PlanetMasses[j] / Dist[j] / Dist[j] / Dist[j] * (y[j] - y[i]);
        }
      }
    }
    for (int i = 0; i < 4 * nb; i++) deriv[i] *= dt;
  }
  void RungeKutta(const double *q0, double timestep, const double *PlanetMasses, double *q1, int nb,
                  const int *feelothers) {
    int n4 = 4 * nb;
    std::vector<double> k1(n4, 0.0), k2(n4, 0.0), k3(n4, 0.0), k4(n4, 0.0), k5(n4, 0.0), k6(n4, 0.0);
    auto translate = [&](double c1, double c2, double c3, double c4, double c5) {
      for (int i = 0; i < n4; i++) q1[i] = q0[i] + c1 * k1[i] + c2 * k2[i] + c3 * k3[i] + c4 * k4[i] + c5 * k5[i];
    };
    DerivMotionRK5(q0, PlanetMasses, k1.data(), nb, timestep, feelothers);
    translate(0.2, 0.0, 0.0, 0.0, 0.0);
    DerivMotionRK5(q1, PlanetMasses, k2.data(), nb, timestep, feelothers);
    translate(0.075, 0.225, 0.0, 0.0, 0.0);
    DerivMotionRK5(q1, PlanetMasses, k3.data(), nb, timestep, feelothers);
    translate(0.3, -0.9, 1.2, 0.0, 0.0);
    DerivMotionRK5(q1, PlanetMasses, k4.data(), nb, timestep, feelothers);
    translate(-11.0 / 54.0, 2.5, -70.0 / 27.0, 35.0 / 27.0, 0.0);
    DerivMotionRK5(q1, PlanetMasses, k5.data(), nb, timestep, feelothers);
    translate(1631.0 / 55296.0, 175.0 / 512.0, 575.0 / 13824.0, 44275.0 / 110592.0, 253.0 / 4096.0);
    DerivMotionRK5(q1, PlanetMasses, k6.data(), nb, timestep, feelothers);
    for (int i = 0; i < n4; i++)
      q1[i] = q0[i] + 37.0 / 378.0 * k1[i] + 250.0 / 621.0 * k3[i] + 125.0 / 594.0 * k4[i] + 512.0 / 1771.0 * k6[i];
  }
  /* AdvanceSystemRK5 src/Pframeforce.cu:124-187 */
  void AdvanceSystemRK5(double dt) {
    int nb = sys.nb;
    std::vector<double> q0(4 * nb + 4, 0.0), q1(4 * nb + 4, 0.0), PlanetMasses(nb + 1, 0.0);
    if (!P.forced_circular) {
      for (int k = 0; k < nb; k++) {
        q0[k] = sys.x[k]; q0[k + nb] = sys.y[k]; q0[k + 2 * nb] = sys.vx[k]; q0[k + 3 * nb] = sys.vy[k];
        PlanetMasses[k] = sys.mass[k];
      }
      if (nb > 0) RungeKutta(q0.data(), dt, PlanetMasses.data(), q1.data(), nb, sys.feelothers.data());
    }
    for (int i = 1 - (PhysicalTime >= P.releasedate); i < sys.nb; i++) {
      if (!P.forced_circular) {
        sys.x[i] = q1[i]; sys.y[i] = q1[i + nb]; sys.vx[i] = q1[i + 2 * nb]; sys.vy[i] = q1[i + 3 * nb];
      } else {
        double x = sys.x[i], y = sys.y[i];
        double theta = atan2(y, x);
        double vx = sys.vx[i], vy = sys.vy[i];
        double r = sqrt(x * x + y * y);
        double omega = (-y * vx + x * vy) / r / r;
        double dtheta = omega * dt;
        sys.x[i] = r * cos(theta + dtheta);
        sys.y[i] = r * sin(theta + dtheta);
        sys.vx[i] = vx * cos(dtheta + theta) - vy * sin(dtheta + theta);
        sys.vy[i] = vx * sin(dtheta + theta) + vy * cos(dtheta + theta);
      }
    }
    if (PhysicalTime < P.releasedate && sys.nb > 0) {
      double x = sys.x[0], y = sys.y[0];
      double r = sqrt(x * x + y * y);
      double theta = atan2(y, x);
      double rdot = (P.releaseradius - r) / (P.releasedate - PhysicalTime);
      double omega = sqrt((1. + sys.mass[0]) / r / r / r);
      double new_r = r + rdot * dt;
      double denom = r - new_r;
      double dtheta;
      if (denom != 0.0) dtheta = 2. * dt * r * omega / denom * (sqrt(r / new_r) - 1.);
      else dtheta = omega * dt;
      double vx = rdot;
      double vy = new_r * sqrt((1. + sys.mass[0]) / new_r / new_r / new_r);
      sys.x[0] = new_r * cos(dtheta + theta);
      sys.y[0] = new_r * sin(dtheta + theta);
      sys.vx[0] = vx * cos(dtheta + theta) - vy * sin(dtheta + theta);
      sys.vy[0] = vx * sin(dtheta + theta) + vx * cos(dtheta + theta);
    }
  }
  /* GetPsysInfo src/Psys.cu:249-319 */
  double GetPsysInfo(int action) {
    double d1, d2, cross, x, y, vx, vy, m, h, d, Ax, Ay, e, a, E, M, xc, yc, vxc, vyc, omega, arg, PerihelionPA;
    xc = x = sys.x[0]; yc = y = sys.y[0]; vxc = vx = sys.vx[0]; vyc = vy = sys.vy[0];
    m = sys.mass[0] + 1.;
    h = x * vy - y * vx;
    d = sqrt(x * x + y * y);
    Ax = x * vy * vy - y * vx * vy - G * m * x / d;
    Ay = y * vx * vx - x * vx * vy - G * m * y / d;
    e = sqrt(Ax * Ax + Ay * Ay) / m;
    a = h * h / G / m / (1. - e * e);
    if (e == 0.0) arg = 1.0; else arg = (1.0 - d / a) / e;
    if (fabs(arg) >= 1.0) E = PI * (1. - arg / fabs(arg)) / 2.;
    else E = acos((1.0 - d / a) / e);
    if ((x * y * (vy * vy - vx * vx) + vx * vy * (x * x - y * y)) < 0) E = -E;
    M = E - e * sin(E);
    PerihelionPA = atan2(Ay, Ax);
    omega = sqrt(m / a / a / a);
    if (P.guiding_center == YES) {
      xc = a * cos(M + PerihelionPA);
      yc = a * sin(M + PerihelionPA);
      vxc = -a * omega * sin(M + PerihelionPA);
      vyc = a * omega * cos(M + PerihelionPA);
    }
    if (e < 1e-08) { xc = x; yc = y; vxc = vx; vyc = vy; }
    (void)vxc; (void)vyc;
    switch (action) {
      case 1: XplanetMark = xc; YplanetMark = yc; return 0.;
      case 0:
        x = xc; y = yc;
        d2 = sqrt(x * x + y * y);
        d1 = sqrt(XplanetMark * XplanetMark + YplanetMark * YplanetMark);
        cross = XplanetMark * y - x * YplanetMark;
        XplanetMark = x; YplanetMark = y;
        return asin(cross / (d1 * d2));
      case 2: return omega;
    }
    return 0.0;
  }
  /* RotatePsys src/Psys.cu:323-340 */
  void RotatePsys(double angle) {
    double sint = sin(angle), cost = cos(angle);
    for (int i = 0; i < sys.nb; i++) {
      double xt = sys.x[i], yt = sys.y[i];
      sys.x[i] = xt * cost + yt * sint;
      sys.y[i] = -xt * sint + yt * cost;
      xt = sys.vx[i]; yt = sys.vy[i];
      sys.vx[i] = xt * cost + yt * sint;
      sys.vy[i] = -xt * sint + yt * cost;
    }
  }

  /* ------------------------------------------------------------------ */
  /* ApplyBoundaryCondition src/SideEuler.cu:31-41 */
  void ApplyBoundaryCondition(double step) {
    if (P.open_inner == YES) OpenBoundary();
    if (P.non_reflecting == YES) {
      if (P.adiabatic) ComputeSoundSpeed();
      NonReflectingBoundary();
    }
    if (P.evanescent == YES) EvanescentBoundary(step);
  }
  /* OpenBoundaryKernel src/Kernels.cu:482-495 */
  void OpenBoundary() {
    int i = 1;
    for (int j = 0; j < NSEC; j++) {
      Dens[(size_t)(i - 1) * NSEC + j] = Dens[(size_t)i * NSEC + j];
      Energy[(size_t)(i - 1) * NSEC + j] = Energy[(size_t)i * NSEC + j];
      if (Vrad[(size_t)(i + 1) * NSEC + j] > 0.0 || (Dens[(size_t)i * NSEC + j] < SigmaMed[0]))
        Vrad[(size_t)i * NSEC + j] = 0.0;
      else
        Vrad[(size_t)i * NSEC + j] = Vrad[(size_t)(i + 1) * NSEC + j];
    }
  }
  /* NonReflectingBoundary src/SideEuler.cu:45-76 + kernels src/Kernels.cu:498-607.
     NonReflectingBoundaryKernel2 has no j < nsec guard: its nsec2pot threads write
     past ring 1 (into ring 2) and past ring nrad-1 (into ring nrad); threads run in
     increasing j here, as in a sequential execution of the launch. */
  void NonReflectingBoundary() {
    std::vector<double> tmp(NSEC);
    for (int j = 0; j < NSEC; j++) tmp[j] = SoundSpeed[j];
    double cs0_r = device_reduce(tmp.data(), NSEC) / NSEC;
    for (int j = 0; j < NSEC; j++) tmp[j] = SoundSpeed[(size_t)NSEC + j];
    double cs1_r = device_reduce(tmp.data(), NSEC) / NSEC;
    for (int j = 0; j < NSEC; j++) tmp[j] = SoundSpeed[(size_t)(NRAD - 1) * NSEC + j];
    double csnrm1_r = device_reduce(tmp.data(), NSEC) / NSEC;
    for (int j = 0; j < NSEC; j++) tmp[j] = SoundSpeed[(size_t)(NRAD - 2) * NSEC + j];
    double csnrm2_r = device_reduce(tmp.data(), NSEC) / NSEC;
    int i = 1;
    double dangle = (pow(Rinf[i], -1.5) - 1.0) / (.5 * (cs0_r + cs1_r));
    dangle *= (Rmed[i] - Rmed[i - 1]);
    int i_angle = (int)(dangle / 2.0 / PI * (double)NSEC + .5);
    i = NRAD - 1;
    double dangle2 = (pow(Rinf[i - 1], -1.5) - 1.0) / (.5 * (csnrm1_r + csnrm2_r));
    dangle2 *= (Rmed[i] - Rmed[i - 1]);
    int i_angle2 = (int)(dangle2 / 2.0 / PI * (double)NSEC + .5);
    double SigmaMed1 = SigmaMed[1], SigmaMed2 = SigmaMed[NRAD - 2];
    /* NonReflectingBoundaryKernel (guarded by j < nsec): sources are rings 1 and
       nrad-2, targets rings 0 and nrad-1 */
    for (int j = 0; j < NSEC; j++) {
      int ii = 1;
      long tgt;
      if (j + i_angle >= NSEC) tgt = j + i_angle - NSEC;
      else if (j + i_angle < 0) tgt = j + i_angle + NSEC;
      else tgt = j + i_angle;
      Dens[tgt] = Dens[(size_t)ii * NSEC + j];
      Energy[tgt] = Energy[(size_t)ii * NSEC + j];
    }
    for (int j = 0; j < NSEC; j++) {
      long ii = NRAD - 1;
      long src;
      if (j - i_angle2 >= NSEC) src = j - i_angle2 + (ii - 2) * NSEC;
      else if (j - i_angle2 < 0) src = j - i_angle2 + ii * NSEC;
      else src = j - i_angle2 + (ii - 1) * NSEC;
      Dens[ii * NSEC + j] = Dens[src];
      Energy[ii * NSEC + j] = Energy[src];
    }
    /* NonReflectingBoundaryKernel2 */
    for (long j = 0; j < nsec2pot; j++) {
      long ii = 1;
      double Vrad_med = -SoundSpeed[ii * NSEC + j] * (Dens[ii * NSEC + j] - SigmaMed1) / SigmaMed1;
      Vrad[ii * NSEC + j] = 2.0 * Vrad_med - Vrad[(ii + 1) * NSEC + j];
      ii = NRAD - 1;
      Vrad_med = SoundSpeed[ii * NSEC + j] * (Dens[(ii - 1) * NSEC + j] - SigmaMed2) / SigmaMed2;
      Vrad[ii * NSEC + j] = 2. * Vrad_med - Vrad[(ii - 1) * NSEC + j];
    }
    /* ReduceMean + MinusMeanKernel */
    for (int j = 0; j < NSEC; j++) tmp[j] = Dens[j];
    double mean_dens_r = device_reduce(tmp.data(), NSEC) / NSEC;
    for (int j = 0; j < NSEC; j++) tmp[j] = Dens[(size_t)(NRAD - 1) * NSEC + j];
    double mean_dens_r2 = device_reduce(tmp.data(), NSEC) / NSEC;
    for (int j = 0; j < NSEC; j++) tmp[j] = Energy[j];
    double mean_energy_r = device_reduce(tmp.data(), NSEC) / NSEC;
    for (int j = 0; j < NSEC; j++) tmp[j] = Energy[(size_t)(NRAD - 1) * NSEC + j];
    double mean_energy_r2 = device_reduce(tmp.data(), NSEC) / NSEC;
    for (int j = 0; j < NSEC; j++) {
      Dens[j] += SigmaMed[0] - mean_dens_r;
      Energy[j] += EnergyMed[0] - mean_energy_r;
      Dens[(size_t)(NRAD - 1) * NSEC + j] += SigmaMed[NRAD - 1] - mean_dens_r2;
      Energy[(size_t)(NRAD - 1) * NSEC + j] += EnergyMed[NRAD - 1] - mean_energy_r2;
    }
  }
  /* EvanescentBoundary src/SideEuler.cu:104-123; kernel src/Kernels.cu:967-1015.
     GLOBAL_bufarray_d is never written on the device (Make1Dprofile copies to the
     host array only, src/Kernels.cu:643), so its SG term reads zero. */
  void EvanescentBoundary(double step) {
    double Tin = 2.0 * PI * pow(Rmed[0], 3. / 2);
    double Tout = 2.0 * PI * pow(Rmed[NRAD - 1], 3. / 2);
    double DRMIN = Rmed[0] * 1.25;
    double DRMAX = Rmed[NRAD - 1] * 0.84;
    for (int i = 0; i < NRAD; i++) viscosity_array[i] = FViscosity(Rmed[i]);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++) {
      if (!((Rmed[i] < DRMIN) || (Rmed[i] > DRMAX))) continue;
      double damping = 0.0, lambda = 0.0, vtheta0, vrad0, energy0, dens0, AR;
      if (Rmed[i] < DRMIN) {
        damping = (Rmed[i] - DRMIN) / (Rmed[0] - DRMIN);
        lambda = damping * damping * 10.0 * step / Tin;
      }
      if (Rmed[i] > DRMAX) {
        damping = (Rmed[i] - DRMAX) / (Rmed[NRAD - 1] - DRMAX);
        lambda = damping * damping * 10.0 * step / Tout;
      }
      AR = AspectRatio(Rmed[i]);
      if (!P.self_gravity)
        vtheta0 = sqrt(G * 1.0 / Rmed[i] *
                       (1.0 - (1.0 + P.sigmaslope - 2.0 * P.flaringindex) * pow(AR, 2.0) * pow(Rmed[i], 2.0 * P.flaringindex)));
      else
        vtheta0 = sqrt(G * 1.0 / Rmed[i] *
                           (1.0 - (1.0 + P.sigmaslope - 2.0 * P.flaringindex) * pow(AR, 2.0) *
                                      pow(Rmed[i], 2.0 * P.flaringindex)) -
                       Rmed[i] * 0.0);
      vtheta0 -= Rmed[i] * OmegaFrame;
      vrad0 = -3.0 * viscosity_array[i] / Rmed[i] * (-P.sigmaslope + .5);
      dens0 = SigmaMed[i];
      energy0 = EnergyMed[i];
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        Vrad[c] = (Vrad[c] + lambda * vrad0) / (1.0 + lambda);
        Vtheta[c] = (Vtheta[c] + lambda * vtheta0) / (1.0 + lambda);
        Dens[c] = (Dens[c] + lambda * dens0) / (1.0 + lambda);
        if (P.adiabatic) Energy[c] = (Energy[c] + lambda * energy0) / (1.0 + lambda);
      }
    }
  }
  /* ApplySubKeplerianBoundary src/SideEuler.cu:189-213; kernel src/Kernels.cu:1416-1430 */
  void ApplySubKeplerianBoundary() {
    double VKepIn, VKepOut;
    if (!P.self_gravity) {
      VKepIn = sqrt(G * 1.0 / Rmed[0] *
                    (1.0 - (1.0 + P.sigmaslope - 2.0 * P.flaringindex) * pow(AspectRatio(Rmed[0]), 2.0) *
                               pow(Rmed[0], 2.0 * P.flaringindex)));
      VKepOut = sqrt(G * 1.0 / Rmed[NRAD - 1] *
                     (1.0 - (1.0 + P.sigmaslope - 2.0 * P.flaringindex) * pow(AspectRatio(Rmed[NRAD - 1]), 2.0) *
                                pow(Rmed[NRAD - 1], 2.0 * P.flaringindex)));
    } else {
      Make1Dprofile_cs();
      for (int i = 0; i < NRAD; i++) GLOBAL_AxiSGAccr[i] = GLOBAL_bufarray[i];
      VKepIn = sqrt(G * 1.0 / Rmed[0] *
                        (1.0 - (1.0 + P.sigmaslope - 2.0 * P.flaringindex) * pow(AspectRatio(Rmed[0]), 2.0) *
                                   pow(Rmed[0], 2.0 * P.flaringindex)) -
                    Rmed[0] * GLOBAL_AxiSGAccr[0]);
      VKepOut = sqrt(G * 1.0 / Rmed[NRAD - 1] *
                         (1.0 - (1.0 + P.sigmaslope - 2.0 * P.flaringindex) * pow(AspectRatio(Rmed[NRAD - 1]), 2.0) *
                                    pow(Rmed[NRAD - 1], 2.0 * P.flaringindex)) -
                     Rmed[NRAD - 1] * GLOBAL_AxiSGAccr[NRAD - 1]);
    }
    for (int j = 0; j < NSEC; j++) {
      VthetaInt[j] = VKepIn - Rmed[0] * OmegaFrame;
      VthetaInt[(size_t)(NRAD - 1) * NSEC + j] = VKepOut - Rmed[NRAD - 1] * OmegaFrame;
    }
  }

  /* ------------------------------------------------------------------ */
  /* Substep1 src/SourceEuler.cu:311-341; Substep1Kernel src/Kernels.cu:13-53 */
  void Substep1(double dt) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++) {
      double supp_torque = P.imposeddiskdrift * 0.5 * pow(Rmed[i], -2.5 + P.sigmaslope);
      double dxtheta = 2.0 * PI / (double)NSEC * Rmed[i];
      double invdxtheta = 1.0 / dxtheta;
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        if (i > 0) {
          double gradp = (Pressure[c] - Pressure[c - NSEC]) * 2.0 / (Dens[c] + Dens[c - NSEC]) * invdiffRmed[i];
          double gradphi = (Potential[c] - Potential[c - NSEC]) * invdiffRmed[i];
          double vt2 = Vtheta[c] + Vtheta[(size_t)i * NSEC + (j + 1) % NSEC] + Vtheta[c - NSEC] +
                       Vtheta[(size_t)(i - 1) * NSEC + (j + 1) % NSEC];
          vt2 = vt2 / 4.0 + OmegaFrame * Rinf[i];
          vt2 = vt2 * vt2;
          double vradint = -gradp - gradphi;
          double vradint2 = vradint + vt2 * invRinf[i];
          VradInt[c] = Vrad[c] + dt * vradint2;
        }
        size_t cm = (size_t)i * NSEC + ((j - 1) + NSEC) % NSEC;
        double gradp = (Pressure[c] - Pressure[cm]) * 2.0 / (Dens[c] + Dens[cm]) * invdxtheta;
        double gradphi = (Potential[c] - Potential[cm]) * invdxtheta;
        VthetaInt[c] = Vtheta[c] - dt * (gradp + gradphi);
        VthetaInt[c] += dt * supp_torque;
      }
    }
    if (P.self_gravity) compute_selfgravity(dt, true);
    ComputeViscousTerms(VradInt, VthetaInt);
    UpdateVelocitiesWithViscosity(dt);
    if (!P.evanescent) ApplySubKeplerianBoundary();
  }

  /* ComputeViscousTerms src/Viscosity.cu:52-67; ViscousTermsKernel src/Kernels.cu:733-771 */
  void ComputeViscousTerms(const vec &Vradial, const vec &Vazimutal) {
    if (P.viscosity_alpha) Make1Dprofile_cs();
    for (int i = 0; i < NRAD; i++) viscosity_array[i] = FViscosity(Rmed[i]);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++) {
      double dphi = 2.0 * M_PI / (double)NSEC;
      double invdphi = 1.0 / dphi;
      double onethird = 1.0 / 3.0;
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        size_t cp = (size_t)i * NSEC + (j + 1) % NSEC;
        size_t cm = (size_t)i * NSEC + ((j - 1) + NSEC) % NSEC;
        DRR[c] = (Vradial[c + NSEC] - Vradial[c]) * invdiffRsup[i];
        DPP[c] = (Vazimutal[cp] - Vazimutal[c]) * invdphi * invRmed[i] + 0.5 * (Vradial[c + NSEC] + Vradial[c]) * invRmed[i];
        DivergenceVelocity[c] = (Vradial[c + NSEC] * Rsup[i] - Vradial[c] * Rinf[i]) * invdiffRsup[i] * invRmed[i];
        DivergenceVelocity[c] += (Vazimutal[cp] - Vazimutal[c]) * invdphi * invRmed[i];
        if (i > 0)
          DRP[c] = 0.5 * (Rinf[i] * (Vazimutal[c] * invRmed[i] - Vazimutal[c - NSEC] * invRmed[i - 1]) * invdiffRmed[i] +
                          (Vradial[c] - Vradial[cm]) * invdphi * invRinf[i]);
        TAURR[c] = 2.0 * Dens[c] * viscosity_array[i] * (DRR[c] - onethird * DivergenceVelocity[c]);
        TAUPP[c] = 2.0 * Dens[c] * viscosity_array[i] * (DPP[c] - onethird * DivergenceVelocity[c]);
        if (i > 0)
          TAURP[c] = 2.0 * 0.25 * (Dens[c] + Dens[c - NSEC] + Dens[cm] + Dens[cm - NSEC]) * viscosity_array[i] * DRP[c];
      }
    }
  }

  /* UpdateVelocitiesKernel src/Kernels.cu:118-150 */
  void UpdateVelocitiesWithViscosity(double DeltaT) {
#pragma omp parallel for schedule(static)
    for (int i = 1; i < NRAD; i++) {
      double dphi = 2.0 * M_PI / (double)NSEC;
      double invdphi = 1.0 / dphi;
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        size_t cm = (size_t)i * NSEC + ((j - 1) + NSEC) % NSEC;
        size_t cp = (size_t)i * NSEC + (j + 1) % NSEC;
        if (i < NRAD - 1)
          VthetaInt[c] += DeltaT * invRmed[i] *
                          ((Rsup[i] * TAURP[c + NSEC] - Rinf[i] * TAURP[c]) * invdiffRsup[i] +
                           (TAUPP[c] - TAUPP[cm]) * invdphi + 0.5 * (TAURP[c] + TAURP[c + NSEC])) /
                          (0.5 * (Dens[c] + Dens[cm]));
        VradInt[c] += DeltaT * invRinf[i] *
                      ((Rmed[i] * TAURR[c] - Rmed[i - 1] * TAURR[c - NSEC]) * invdiffRmed[i] +
                       (TAURP[cp] - TAURP[c]) * invdphi - 0.5 * (TAUPP[c] + TAUPP[c - NSEC])) /
                      (0.5 * (Dens[c] + Dens[c - NSEC]));
      }
    }
  }

  /* Substep2 + host src/SourceEuler.cu:345-358; kernels src/Kernels.cu:409-479 */
  void Substep2(double dt) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        double dv = VradInt[c + NSEC] - VradInt[c];
        if (dv < 0.0) DensInt[c] = CVNR * CVNR * Dens[c] * dv * dv;
        else DensInt[c] = 0.0;
        dv = VthetaInt[(size_t)i * NSEC + (j + 1) % NSEC] - VthetaInt[c];
        if (dv < 0.0) TemperInt[c] = CVNR * CVNR * Dens[c] * dv * dv;
        else TemperInt[c] = 0.0;
      }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++) {
      double dxtheta = 2.0 * PI / (double)NSEC * Rmed[i];
      double invdxtheta = 1.0 / dxtheta;
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        size_t cm = (size_t)i * NSEC + ((j - 1) + NSEC) % NSEC;
        if (i > 0) {
          double dens = Dens[c] + Dens[c - NSEC];
          double densint = DensInt[c] - DensInt[c - NSEC];
          VradNew[c] = VradInt[c] - dt * 2.0 / dens * densint * invdiffRmed[i];
        }
        double dens2 = Dens[c] + Dens[cm];
        double tempint = (TemperInt[c] - TemperInt[cm]);
        VthetaNew[c] = VthetaInt[c] - dt * 2.0 / dens2 * tempint * invdxtheta;
        if (P.adiabatic)
          EnergyInt[c] = Energy[c] - dt * DensInt[c] * (VradInt[c + NSEC] - VradInt[c]) * invdiffRsup[i] -
                         dt * TemperInt[c] * (VthetaInt[(size_t)i * NSEC + (j + 1) % NSEC] - VthetaInt[c]) * invdxtheta;
      }
    }
  }

  /* Substep3 src/SourceEuler.cu:362-375; kernels src/Kernels.cu:56-115 */
  void Substep3(double dt) {
    for (int i = 0; i < NRAD; i++) viscosity_array[i] = FViscosity(Rmed[i]);
#pragma omp parallel for schedule(static)
    for (int i = 1; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        if (viscosity_array[i] != 0.0) {
          Qplus[c] = 0.5 / viscosity_array[i] / Dens[c] * (TAURR[c] * TAURR[c] + TAURP[c] * TAURP[c] + TAUPP[c] * TAUPP[c]);
          Qplus[c] += (2.0 / 9.0) * viscosity_array[i] * Dens[c] * DivergenceVelocity[c] * DivergenceVelocity[c];
        } else
          Qplus[c] = 0.0;
      }
    for (int j = 0; j < NSEC; j++) {
      if (viscosity_array[NRAD - 1] != 0.0)
        Qplus[j] = Qplus[(size_t)NSEC + j] * exp(log(Qplus[(size_t)NSEC + j] / Qplus[(size_t)2 * NSEC + j]) *
                                                 log(Rmed[0] / Rmed[1]) / log(Rmed[1] / Rmed[2]));
      else
        Qplus[j] = 0.0;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        double num, den;
        if (!P.cooling) {
          num = dt * Qplus[c] + EnergyInt[c];
          den = 1.0 + (P.adiabaticindex - 1.0) * dt * DivergenceVelocity[c];
          EnergyNew[c] = num / den;
        } else {
          num = EnergyMed[i] * dt * Dens[c] / SigmaMed[i] + CoolingTimeMed[i] * EnergyInt[c] +
                dt * CoolingTimeMed[i] * (Qplus[c] - QplusMed[i] * Dens[c] / SigmaMed[i]);
          den = dt + CoolingTimeMed[i] + (P.adiabaticindex - 1.0) * dt * CoolingTimeMed[i] * DivergenceVelocity[c];
          EnergyNew[c] = num / den;
        }
      }
  }

  /* ------------------------------------------------------------------ */
  /* Transport src/TransportEuler.cu:30-41 */
  void Transport(double dt) {
    /* LRMomentaKernel src/Kernels.cu:774-787 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        RadMomP[c] = Dens[c] * Vrad[c + NSEC];
        RadMomM[c] = Dens[c] * Vrad[c];
        ThetaMomP[c] = Dens[c] * (Vtheta[(size_t)i * NSEC + (j + 1) % NSEC] + Rmed[i] * OmegaFrame) * Rmed[i];
        ThetaMomM[c] = Dens[c] * (Vtheta[c] + Rmed[i] * OmegaFrame) * Rmed[i];
      }
    OneWindRad(dt);
    OneWindTheta(dt);
    /* ComputeVelocitiesKernel src/Kernels.cu:1193-1210 */
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        size_t cm = (size_t)i * NSEC + ((j - 1) + NSEC) % NSEC;
        if (i == 0) Vrad[c] = 0.0;
        else Vrad[c] = (RadMomP[c - NSEC] + RadMomM[c]) / (Dens[c] + Dens[c - NSEC] + 1e-20);
        Vtheta[c] = (ThetaMomP[cm] + ThetaMomM[c]) / (Dens[c] + Dens[cm] + 1e-15) / Rmed[i] - Rmed[i] * OmegaFrame;
      }
  }

  /* StarRadKernel + StarRadKernel2 src/Kernels.cu:800-838 */
  void ComputeStarRad(const vec &Qbase2, vec &QStar, double dt) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        if (i == 0 || i == NRAD - 1) dq[i + (size_t)j * NRAD] = 0.0;
        else {
          double dqm = (Qbase2[c] - Qbase2[c - NSEC]) * invdiffRmed[i];
          double dqp = (Qbase2[c + NSEC] - Qbase2[c]) * invdiffRmed[i + 1];
          if (dqp * dqm > 0.0) dq[i + (size_t)j * NRAD] = 2.0 * dqp * dqm / (dqp + dqm);
          else dq[i + (size_t)j * NRAD] = 0.0;
        }
      }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        if (Vrad[c] > 0.0 && i > 0)
          QStar[c] = Qbase2[c - NSEC] + (Rmed[i] - Rmed[i - 1] - Vrad[c] * dt) * 0.5 * dq[i - 1 + (size_t)j * NRAD];
        else
          QStar[c] = Qbase2[c] - (Rmed[i + 1] - Rmed[i] + Vrad[c] * dt) * 0.5 * dq[i + (size_t)j * NRAD];
      }
    for (int j = 0; j < NSEC; j++) QStar[j] = QStar[j + (size_t)NSEC * NRAD] = 0.0;
  }
  /* DivisePolarGridKernel src/Kernels.cu:1018-1025 (rings 0..nrad-1) */
  void DivisePolarGrid(const vec &Qbase) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        Work[c] = Qbase[c] / (DensInt[c] + 1e-20);
      }
  }
  /* VanLeerRadial src/TransportEuler.cu:106-156; kernel src/Kernels.cu:1028-1046 */
  double VanLeerRadial(vec &Qbase, double dt, int ReturnLost) {
    DivisePolarGrid(Qbase);
    ComputeStarRad(Work, QRStar, dt);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++) {
      double dtheta = 2.0 * PI / (double)NSEC;
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        double varq = dt * dtheta * Rinf[i] * QRStar[c] * DensStar[c] * Vrad[c];
        varq -= dt * dtheta * Rsup[i] * QRStar[c + NSEC] * DensStar[c + NSEC] * Vrad[c + NSEC];
        Qbase[c] += varq * invSurf[i];
        if (i == 0 && P.open_inner) LostByDisk[j] = varq;
      }
    }
    double Lost = 0.0;
    if (ReturnLost) Lost = device_reduce(LostByDisk.data(), NSEC);
    return Lost;
  }
  /* OneWindRad src/TransportEuler.cu:60-79 */
  void OneWindRad(double dt) {
    ComputeStarRad(Dens, DensStar, dt);
    DensInt = Dens;
    VanLeerRadial(RadMomP, dt, 0);
    VanLeerRadial(RadMomM, dt, 0);
    VanLeerRadial(ThetaMomP, dt, 0);
    VanLeerRadial(ThetaMomM, dt, 0);
    if (P.adiabatic) VanLeerRadial(Energy, dt, 0);
    LostMass += VanLeerRadial(Dens, dt, 1);
  }
  /* StarThetaKernel + StarThetaKernel2 src/Kernels.cu:1129-1170 */
  void ComputeStarTheta(const vec &Qbase, const vec &Vazimutal, vec &QStar, double dt) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++) {
      double dxtheta = 2.0 * PI / (double)NSEC * Rmed[i];
      double invdxtheta = 1.0 / dxtheta;
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        double dqm = (Qbase[c] - Qbase[(size_t)i * NSEC + ((j - 1) + NSEC) % NSEC]);
        double dqp = (Qbase[(size_t)i * NSEC + (j + 1) % NSEC] - Qbase[c]);
        if (dqp * dqm > 0.0) dq[c] = dqp * dqm / (dqp + dqm) * invdxtheta;
        else dq[c] = 0.0;
      }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++) {
      double dxtheta = 2.0 * PI / (double)NSEC * Rmed[i];
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        size_t cm = (size_t)i * NSEC + ((j - 1) + NSEC) % NSEC;
        double ksi = Vazimutal[c] * dt;
        if (ksi > 0.0) QStar[c] = Qbase[cm] + (dxtheta - ksi) * dq[cm];
        else QStar[c] = Qbase[c] - (dxtheta + ksi) * dq[c];
      }
    }
  }
  /* VanLeerTheta src/TransportEuler.cu:249-257; kernel src/Kernels.cu:1049-1066
     (UniformTransport is passed as 0, so the update always runs) */
  void VanLeerTheta(const vec &Vazimutal, vec &Qbase, double dt) {
    DivisePolarGrid(Qbase);
    ComputeStarTheta(Work, Vazimutal, QRStar, dt);
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++) {
      double dxrad = (Rsup[i] - Rinf[i]) * dt;
      double invsurf = 1.0 / Surf[i];
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        size_t cp = (size_t)i * NSEC + (j + 1) % NSEC;
        double varq = dxrad * QRStar[c] * DensStar[c] * Vazimutal[c];
        varq -= dxrad * QRStar[cp] * DensStar[cp] * Vazimutal[cp];
        Qbase[c] += varq * invsurf;
      }
    }
  }
  /* QuantitiesAdvection src/TransportEuler.cu:229-245 */
  void QuantitiesAdvection(const vec &Vazimutal, double dt) {
    ComputeStarTheta(Dens, Vazimutal, DensStar, dt);
    DensInt = Dens;
    VanLeerTheta(Vazimutal, RadMomP, dt);
    VanLeerTheta(Vazimutal, RadMomM, dt);
    VanLeerTheta(Vazimutal, ThetaMomP, dt);
    VanLeerTheta(Vazimutal, ThetaMomM, dt);
    if (P.adiabatic) VanLeerTheta(Vazimutal, Energy, dt);
    VanLeerTheta(Vazimutal, Dens, dt);
  }
  /* AdvectSHIFT src/TransportEuler.cu:210-216; kernel src/Kernels.cu:1173-1190
     (the copy-back of the whole TempShift buffer zeroes ring nrad) */
  void AdvectSHIFT(vec &a) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) {
        int ji = j - Nshift[i];
        while (ji < 0) ji += NSEC;
        while (ji >= NSEC) ji -= NSEC;
        TempShift[(size_t)i * NSEC + j] = a[(size_t)i * NSEC + ji];
      }
    a = TempShift;
  }
  /* OneWindTheta src/TransportEuler.cu:177-194 */
  void OneWindTheta(double dt) {
    /* ComputeAverageThetaVelocitiesKernel src/Kernels.cu:1070-1081 */
    for (int i = 0; i < NRAD; i++) {
      double moy = 0.0;
      for (int j = 0; j < NSEC; j++) moy += Vtheta[(size_t)i * NSEC + j];
      VMed[i] = moy / (double)NSEC;
    }
    /* ComputeResidualsKernel src/Kernels.cu:1084-1091 */
    for (int i = 0; i < NRAD; i++)
      for (int j = 0; j < NSEC; j++) VthetaRes[(size_t)i * NSEC + j] = Vtheta[(size_t)i * NSEC + j] - VMed[i];
    /* ComputeConstantResidualKernel src/Kernels.cu:1094-1126 */
    for (int i = 0; i < NRAD; i++) {
      double maxfrac = P.fast_transport ? 1.0 : 0.0;
      double invdt = 1.0 / dt;
      double dpinvns = 2.0 * PI / (double)NSEC;
      double Ntilde = VMed[i] * invRmed[i] * dt * (double)NSEC / 2.0 / PI;
      double Nround = floor(Ntilde + 0.5);
      long nitemp = (long)Nround;
      Nshift[i] = (int)(long)nitemp;
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        Vtheta[c] = (Ntilde - Nround) * Rmed[i] * invdt * dpinvns;
        if (maxfrac < 0.5) {
          NoSplitAdvection[i] = YES;
          VthetaRes[c] += Vtheta[c];
          Vtheta[c] = 0.0;
        } else
          NoSplitAdvection[i] = NO;
      }
    }
    QuantitiesAdvection(VthetaRes, dt);
    QuantitiesAdvection(Vtheta, dt);
    AdvectSHIFT(RadMomP);
    AdvectSHIFT(RadMomM);
    AdvectSHIFT(ThetaMomP);
    AdvectSHIFT(ThetaMomM);
    if (P.adiabatic) AdvectSHIFT(Energy);
    AdvectSHIFT(Dens);
  }

  /* ------------------------------------------------------------------ */
  /* compute_kernel src/SgMain.cu:49-81 (host, float coshf) */
  void compute_kernel() {
    int n0 = 2 * NRAD;
    Kr_aux.assign((size_t)n0 * NSEC, 0.0);
    Kt_aux.assign((size_t)n0 * NSEC, 0.0);
    for (int i = 0; i < n0; i++) {
      double u;
      if (i < NRAD) u = log(Radii[i] / Radii[0]);
      else u = -log(Radii[2 * NRAD - i] / Radii[0]);
      for (int j = 0; j < NSEC; j++) {
        double theta = 2.0 * PI * (double)j / (double)NSEC;
        double Kr = 1.0 + SGP_eps * SGP_eps - cos(theta) * exp(-u);
        double base = SGP_eps * SGP_eps * exp(u) + 2.0 * (coshf(u) - cos(theta));
        Kr *= pow(base, -1.5);
        double Kt = sin(theta);
        Kt *= pow(base, -1.5);
        Kr_aux[(size_t)i * NSEC + j] = Kr;
        Kt_aux[(size_t)i * NSEC + j] = Kt;
      }
    }
    /* the kernel spectra are recomputed at every call by the reference
       (src/Kernels.cu:849-853, src/SgMain.cu:124,138); they are constant */
    Kr_hat.assign((size_t)n0 * NSEC, fftref::cplx(0, 0));
    Kt_hat.assign((size_t)n0 * NSEC, fftref::cplx(0, 0));
    for (size_t c = 0; c < (size_t)n0 * NSEC; c++) {
      Kr_hat[c] = fftref::cplx(Kr_aux[c], 0.);
      Kt_hat[c] = fftref::cplx(Kt_aux[c], 0.);
    }
    fftref::fft2d(Kr_hat.data(), n0, NSEC, -1);
    fftref::fft2d(Kt_hat.data(), n0, NSEC, -1);
  }
  /* compute_selfgravity src/SgMain.cu:23-45; kernels src/Kernels.cu:840-932 */
  void compute_selfgravity(double DeltaT, bool SGUpdate) {
    int n0 = 2 * NRAD;
    size_t nt = (size_t)n0 * NSEC;
    std::vector<fftref::cplx> Sr(nt), St(nt), Gr(nt), Gphi(nt);
    for (int i = 0; i < n0; i++)
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        if (i < NRAD) {
          double var = Dens[c] * sqrt(Rmed[i] / Rmed[0]);
          Sr[c] = fftref::cplx(var, 0.);
          St[c] = fftref::cplx(var * Rmed[i] / Rmed[0], 0.);
        } else {
          Sr[c] = fftref::cplx(0., 0.);
          St[c] = fftref::cplx(0., 0.);
        }
      }
    fftref::fft2d(St.data(), n0, NSEC, -1);
    fftref::fft2d(Sr.data(), n0, NSEC, -1);
    for (size_t c = 0; c < nt; c++) {
      double gpx = -G * (Kt_hat[c].real() * St[c].real() - Kt_hat[c].imag() * St[c].imag());
      double gpy = -G * (Kt_hat[c].real() * St[c].imag() + Kt_hat[c].imag() * St[c].real());
      double grx = -G * (Kr_hat[c].real() * Sr[c].real() - Kr_hat[c].imag() * Sr[c].imag());
      double gry = -G * (Kr_hat[c].real() * Sr[c].imag() + Kr_hat[c].imag() * Sr[c].real());
      Gphi[c] = fftref::cplx(gpx, gpy);
      Gr[c] = fftref::cplx(grx, gry);
    }
    fftref::fft2d(Gphi.data(), n0, NSEC, +1);
    fftref::fft2d(Gr.data(), n0, NSEC, +1);
    for (int i = 0; i < NRAD; i++) {
      double divRmed = Rmed[i] / Rmed[0];
      double normaccr = SGP_rstep * SGP_tstep / ((double)(2 * NRAD) * (double)NSEC);
      double normacct = normaccr;
      normaccr /= sqrt(divRmed);
      normacct /= (divRmed * sqrt(divRmed));
      for (int j = 0; j < NSEC; j++) {
        size_t c = (size_t)i * NSEC + j;
        SG_Acct[c] = Gphi[c].real() * normacct;
        SG_Accr[c] = Gr[c].real() * normaccr;
        SG_Accr[c] += G * Dens[c] * SGP_rstep * SGP_tstep / SGP_eps;
      }
    }
    if (SGUpdate) {
      /* Update_sgvelocityKernel src/Kernels.cu:915-932 on VradInt / VthetaInt
         (copied through Vradial/Vazimutal, src/SourceEuler.cu:326-332).
         (j-1)%nsec is -1 at j = 0: the flat index i*nsec-1 is the previous ring's
         last cell; at i = 0 it falls before the array and is taken as 0. */
      for (int i = 0; i < NRAD; i++)
        for (int j = 0; j < NSEC; j++) {
          size_t c = (size_t)i * NSEC + j;
          if (i > 0)
            VradInt[c] += DeltaT * ((Rinf[i] - Rmed[i - 1]) * SG_Accr[c] + (Rmed[i] - Rinf[i]) * SG_Accr[c - NSEC]) *
                          invdiffRmed[i];
          long k = (long)i * NSEC + (j - 1) % NSEC;
          double prev = (k >= 0) ? SG_Acct[k] : 0.0;
          VthetaInt[c] += 0.5 * DeltaT * (SG_Acct[c] + prev);
        }
    }
  }
  /* Init_planetarysys_withSG src/SgMain.cu:166-194.  The reference aborts here:
     Make1Dprofile(1) copies from SoundSpeed_d before it is allocated
     (src/Main.cu:289 runs before InitEuler).  The restatement uses the radial
     self-gravity acceleration averaged in azimuth, which is what the comment at
     src/SgMain.cu:175-177 describes. */
  void Init_planetarysys_withSG() {
    for (int i = 0; i < NRAD; i++) {
      double sum = 0.0;
      for (int j = 0; j < NSEC; j++) sum += SG_Accr[(size_t)i * NSEC + j];
      GLOBAL_AxiSGAccr[i] = sum / (double)NSEC;
    }
    for (int k = 0; k < sys.nb; k++) {
      double r = sys.x[k];
      double dist = (double)(r / (1. + P.eccentricity));
      int ipl = 0;
      while (ipl < NRAD - 2 && Rmed[ipl] <= dist) ipl++;
      double ri = Rmed[ipl], rip1 = Rmed[ipl + 1];
      double dr = rip1 - ri;
      double sgacc = (dist - ri) * GLOBAL_AxiSGAccr[ipl + 1] + (rip1 - dist) * GLOBAL_AxiSGAccr[ipl];
      sgacc /= dr;
      sys.vy[k] *= (double)sqrt(1. - dist * dist * sgacc);
    }
  }

  /* ------------------------------------------------------------------ */
  /* One iteration of the AlgoGas while loop, src/SourceEuler.cu:223-302, given dt. */
  void substep_body(double dt) {
    if (P.corotating == YES) GetPsysInfo(1 /* MARK */);
    if (P.is_disk == YES) {
      ComputeAccel(0.0, 0.0, 0.0, &DiskOnPrimaryX, &DiskOnPrimaryY);
      FillForcesArrays();
      AdvanceSystemFromDisk(dt);
    }
    AdvanceSystemRK5(dt);
    if (P.corotating == YES) {
      double OmegaNew = GetPsysInfo(0 /* GET */) / dt;
      double domega = OmegaNew - OmegaFrame;
      if (P.is_disk == YES) {
        for (int i = 0; i < NRAD; i++)
          for (int j = 0; j < NSEC; j++) Vtheta[(size_t)i * NSEC + j] = Vtheta[(size_t)i * NSEC + j] - domega * Rmed[i];
      }
      OmegaFrame = OmegaNew;
    }
    RotatePsys(OmegaFrame * dt);
    if (P.is_disk == YES) {
      ApplyBoundaryCondition(dt);
      ComputePressureField();
      Substep1(dt);
      Substep2(dt);
      /* ActualiseGasVrad / ActualiseGasVtheta (whole buffers) */
      Vrad = VradNew;
      Vtheta = VthetaNew;
      ApplyBoundaryCondition(dt);
      if (P.adiabatic) {
        ComputeViscousTerms(Vrad, Vtheta);
        Substep3(dt);
        Energy = EnergyNew;
      }
      Transport(dt);
      ApplyBoundaryCondition(dt);
      ComputeTemperatureField();
    }
    PhysicalTime += dt;
    last_dt = dt;
    substeps++;
  }

  /* AlgoGas src/SourceEuler.cu:199-307 */
  int AlgoGas(int *nsub) {
    double dt, dtemp = 0.0;
    int gastimestepcfl = 1;
    int n = 0;
    if (P.adiabatic) ComputeSoundSpeed();
    if (P.is_disk == YES && P.sloppy_cfl == YES) gastimestepcfl = ConditionCFL(P.dt - dtemp);
    dt = P.dt / gastimestepcfl;
    while (dtemp < 0.999999999 * P.dt) {
      MassTaper = PhysicalTime / (P.masstaper * 2.0 * M_PI);
      MassTaper = (MassTaper > 1.0 ? 1.0 : pow(sin(MassTaper * M_PI / 2.0), 2.0));
      if (P.is_disk == YES) {
        if (P.sloppy_cfl == NO) {
          gastimestepcfl = 1;
          gastimestepcfl = ConditionCFL(P.dt - dtemp);
          dt = (P.dt - dtemp) / (double)gastimestepcfl;
        }
      }
      last_cfl = gastimestepcfl;
      if (!(dt > 0.0) || !std::isfinite(dt)) { err = "non-positive or non-finite substep"; return FARGO_ERR_NUMERIC; }
      dtemp += dt;
      DiskOnPrimaryX = 0.0;
      DiskOnPrimaryY = 0.0;
      substep_body(dt);
      n++;
      if (n > 1000000) { err = "substep cap exceeded"; return FARGO_ERR_NUMERIC; }
    }
    if (nsub) *nsub = n;
    return FARGO_OK;
  }

  vec *field(int which) {
    switch (which) {
      case FARGO_FIELD_DENS: return &Dens;
      case FARGO_FIELD_VRAD: return &Vrad;
      case FARGO_FIELD_VTHETA: return &Vtheta;
      case FARGO_FIELD_ENERGY: return &Energy;
      case FARGO_FIELD_TEMPERATURE: return &Temperature;
      case FARGO_FIELD_PRESSURE: return &Pressure;
      case FARGO_FIELD_SOUNDSPEED: return &SoundSpeed;
      case FARGO_FIELD_POTENTIAL: return &Potential;
      case FARGO_FIELD_QPLUS: return &Qplus;
      case FARGO_FIELD_DIVERGENCE: return &DivergenceVelocity;
      case FARGO_FIELD_SG_ACCR: return P.self_gravity ? &SG_Accr : nullptr;
      case FARGO_FIELD_SG_ACCT: return P.self_gravity ? &SG_Acct : nullptr;
    }
    return nullptr;
  }
};

}  // namespace

/* ---------------------------------------------------------------------- */
/* C entry points used by the tests and bench.py (ctypes).                 */
extern "C" {

typedef struct orc_ctx orc_ctx;

orc_ctx *orc_create(const fargo_params *p, const fargo_planet *pl, int nb) {
  Oracle *o = new Oracle();
  if (!o->init(p, pl, nb)) { delete o; return nullptr; }
  return (orc_ctx *)o;
}
void orc_destroy(orc_ctx *c) { delete (Oracle *)c; }
const char *orc_last_error(orc_ctx *c) { return ((Oracle *)c)->err.c_str(); }
void orc_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
int orc_get_field(orc_ctx *c, int which, double *out) {
  Oracle *o = (Oracle *)c;
  vec *v = o->field(which);
  if (!v) return FARGO_ERR_INVALID;
  std::memcpy(out, v->data(), sizeof(double) * (size_t)o->size_grid);
  return FARGO_OK;
}
int orc_set_fields(orc_ctx *c, const double *dens, const double *vrad, const double *vtheta, const double *energy) {
  Oracle *o = (Oracle *)c;
  size_t n = (size_t)o->size_grid;
  if (dens) std::memcpy(o->Dens.data(), dens, n * sizeof(double));
  if (vrad) std::memcpy(o->Vrad.data(), vrad, n * sizeof(double));
  if (vtheta) std::memcpy(o->Vtheta.data(), vtheta, n * sizeof(double));
  if (energy) std::memcpy(o->Energy.data(), energy, n * sizeof(double));
  return FARGO_OK;
}
int orc_algogas(orc_ctx *c, int *nsub) { return ((Oracle *)c)->AlgoGas(nsub); }
int orc_condition_cfl(orc_ctx *c, double deltaT, int *cfl) {
  *cfl = ((Oracle *)c)->ConditionCFL(deltaT);
  return FARGO_OK;
}
/* One substep of fixed length dt: the loop body of AlgoGas without the CFL. */
int orc_substep_full(orc_ctx *c, double dt) {
  Oracle *o = (Oracle *)c;
  o->MassTaper = o->PhysicalTime / (o->P.masstaper * 2.0 * M_PI);
  o->MassTaper = (o->MassTaper > 1.0 ? 1.0 : pow(sin(o->MassTaper * M_PI / 2.0), 2.0));
  o->DiskOnPrimaryX = 0.0;
  o->DiskOnPrimaryY = 0.0;
  o->substep_body(dt);
  return FARGO_OK;
}
int orc_substep(orc_ctx *c, int which, double dt) {
  Oracle *o = (Oracle *)c;
  switch (which) {
    case FARGO_SUB_BOUNDARY: o->ApplyBoundaryCondition(dt); break;
    case FARGO_SUB_SOURCE:
      o->ComputePressureField();
      o->Substep1(dt);
      o->Substep2(dt);
      o->Vrad = o->VradNew;
      o->Vtheta = o->VthetaNew;
      break;
    case FARGO_SUB_ENERGY:
      if (!o->P.adiabatic) return FARGO_ERR_INVALID;
      o->ComputeViscousTerms(o->Vrad, o->Vtheta);
      o->Substep3(dt);
      o->Energy = o->EnergyNew;
      break;
    case FARGO_SUB_TRANSPORT: o->Transport(dt); break;
    case FARGO_SUB_TEMPERATURE: o->ComputeTemperatureField(); break;
    case FARGO_SUB_SOUNDSPEED: o->ComputeSoundSpeed(); break;
    case FARGO_SUB_POTENTIAL:
      o->MassTaper = o->PhysicalTime / (o->P.masstaper * 2.0 * M_PI);
      o->MassTaper = (o->MassTaper > 1.0 ? 1.0 : pow(sin(o->MassTaper * M_PI / 2.0), 2.0));
      o->ComputeAccel(0.0, 0.0, 0.0, &o->DiskOnPrimaryX, &o->DiskOnPrimaryY);
      o->FillForcesArrays();
      break;
    default: return FARGO_ERR_INVALID;
  }
  return FARGO_OK;
}
int orc_get_planets(orc_ctx *c, fargo_planet *out, int cap, int *nb) {
  Oracle *o = (Oracle *)c;
  *nb = o->sys.nb;
  for (int k = 0; k < o->sys.nb && k < cap; k++) {
    out[k].x = o->sys.x[k]; out[k].y = o->sys.y[k]; out[k].vx = o->sys.vx[k]; out[k].vy = o->sys.vy[k];
    out[k].mass = o->sys.mass[k]; out[k].acc = o->sys.acc[k];
    out[k].feel_disk = o->sys.feeldisk[k]; out[k].feel_others = o->sys.feelothers[k];
  }
  return FARGO_OK;
}
int orc_get_scalars(orc_ctx *c, fargo_scalars *s) {
  Oracle *o = (Oracle *)c;
  s->physical_time = o->PhysicalTime;
  s->omega_frame = o->OmegaFrame;
  s->lost_mass = o->LostMass;
  s->last_dt = o->last_dt;
  s->substeps = o->substeps;
  s->last_cfl = o->last_cfl;
  s->nb = o->sys.nb;
  return FARGO_OK;
}
int orc_get_mesh(orc_ctx *c, double *rinf, double *rmed, double *rsup, double *surf) {
  Oracle *o = (Oracle *)c;
  size_t n = (size_t)o->NRAD + 1;
  if (rinf) std::memcpy(rinf, o->Rinf.data(), n * sizeof(double));
  if (rmed) std::memcpy(rmed, o->Rmed.data(), n * sizeof(double));
  if (rsup) std::memcpy(rsup, o->Rsup.data(), n * sizeof(double));
  if (surf) std::memcpy(surf, o->Surf.data(), n * sizeof(double));
  return FARGO_OK;
}
/* 2D complex DFT helper, exposed so the tests can pin it against numpy.fft. */
int orc_fft2d(double *re_im, int n0, int n1, int sign) {
  fftref::fft2d((fftref::cplx *)re_im, n0, n1, sign);
  return FARGO_OK;
}
/* DeviceReduce order restatement, exposed for tests. */
double orc_device_reduce(const double *x, int n) { return device_reduce(x, n); }

}  // extern "C"
