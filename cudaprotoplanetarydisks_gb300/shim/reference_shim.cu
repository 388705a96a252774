// reference_shim.cu -- the reference's host driver on this library.
//
// Links the reference's own host-driver objects -- Main (main(), the output
// cadence, its device arrays), Interpret (.par parser), Psys (.cfg planets),
// Output (dumps and planet files), Theo (initial profiles), Init
// (Initialization), LowTasks -- unchanged, against this file and
// libfargo_gb300.so.  This file defines what those objects take from the files the
// library replaces (src/SourceEuler.cu, Pframeforce.cu, Force.cu, SgMain.cu,
// Viscosity.cu, TransportEuler.cu, SideEuler.cu, Kernels.cu): 14 functions and the
// global arrays and scalars, with the types the reference declares.  The hydro
// step itself is the library's (fargo_step_DT = AlgoGas, FP64), created from the
// same .par file the reference's main() reads.
//
// Data flow:
//  * ReadVariables (Interpret.o) is wrapped at link time (--wrap) to learn the .par
//    path; FillPolar1DArrays creates the context from it (same parser semantics,
//    plus the -c / -b switches main() parsed) and fills the 1D mesh arrays that
//    main()'s Cudamalloc copies to the device;
//  * InitGasDensity / InitGasEnergy hand main() the context's initial fields;
//  * AlgoGas advances one DT, copies the planets into the reference's
//    PlanetarySystem and PhysicalTime / LostMass / OmegaFrame into its globals, and
//    the fields into the device arrays main()'s DeviceToHostcudaMemcpy reads
//    (Dens_d, Vrad_d, Vtheta_d, Energy_d, Temperature_d, Qplus_d).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "Main.cuh"  // the reference's declarations (types, prototypes)
#include "fargo_gb300.h"

// ---- globals the kept objects use, defined here (types as the reference declares) ----
double *CellAbscissa, *CellAbscissa_d, *CellOrdinate, *CellOrdinate_d;
double *DPP, *DPP_d, *DRP, *DRP_d, *DRR, *DRR_d, *DT1D_d, *DT2D_d, *newDT_d, *Vmoy_d;
double *DensInt, *DensStar, *DensStar_d, *DivergenceVelocity, *DivergenceVelocity_d;
double *EnergyInt, *EnergyNew, *Energy_d, *ExtLabel, *ExtLabel_d, *Kr_aux, *Kt_aux;
double *LostByDisk_d, *VMed_d, *dq, *dq_d;
int *NoSplitAdvection_d, *Nshift_d;
double LostMass = 0.0, PhysicalTime = 0.0, PhysicalTimeInitial = 0.0;
double exces_mdcp = 0.0, mdcp1 = 0.0;
double *Potential, *Pressure, *Pressure_d, *SoundSpeed, *SoundSpeed_d;
double *QRStar, *QRStar_d, *RadMomM, *RadMomM_d, *RadMomP, *RadMomP_d, *ThetaMomM, *ThetaMomM_d;
double *ThetaMomP, *ThetaMomP_d, *Work, *Work_d, *TempShift, *TempShift_d, *VthetaRes, *VthetaRes_d;
double *Radii, *Rinf, *Rinf_d, *Rmed, *Rsup, *Surf, *invRinf, *invRmed, *invSurf, *invdiffRmed, *invdiffRsup;
double *powRmed, *vt_cent, *vt_cent_d, *SigmaInf_d, *viscosity_array_d;
double *TAUPP, *TAUPP_d, *TAURP, *TAURP_d, *TAURR, *TAURR_d;
double *TemperInt, *TemperInt_d, *Temperature, *Temperature_d;
double *Vazimutal_d, *Vradial_d, *Vresidual_d, *VradInt, *VradInt_d, *VradNew, *Vrad_d;
double *VthetaInt, *VthetaNew, *Vtheta_d;

// ---- globals of the kept objects this file reads or writes ----
extern int NRAD, NSEC, size_grid, Adiabatic, Cooling, SelfGravity, ViscosityAlpha;
extern int SloppyCFL, CentrifugalBalance;
extern double OmegaFrame, *Dens_d, *Qplus_d, *Qplus, *GLOBAL_bufarray;
extern double VISCOSITY, ALPHAVISCOSITY, CAVITYRADIUS, CAVITYWIDTH, CAVITYRATIO, ASPECTRATIO, LAMBDADOUBLING;
extern std::string OUTPUTDIR;

namespace {
fargo_ctx *g_ctx = nullptr;
std::string g_parfile;

[[noreturn]] void fail(const char *what, int rc) {
  std::fprintf(stderr, "%s failed (status %d): %s\n", what, rc, g_ctx ? fargo_last_error(g_ctx) : "no context");
  std::exit(1);
}

void check(int rc, const char *what) {
  if (rc != FARGO_OK) fail(what, rc);
}

double *host_array(size_t n) {
  double *p = (double *)std::calloc(n, sizeof(double));
  if (!p) fail("calloc", FARGO_ERR_INVALID);
  return p;
}

double *device_array(size_t n) {
  double *p = nullptr;
  if (cudaMalloc((void **)&p, n * sizeof(double)) != cudaSuccess || cudaMemset(p, 0, n * sizeof(double)) != cudaSuccess)
    fail("cudaMalloc", FARGO_ERR_CUDA);
  return p;
}

// the fields main()'s DeviceToHostcudaMemcpy copies back, from the context
void publish_fields() {
  check(fargo_get_field_device(g_ctx, FARGO_FIELD_DENS, Dens_d), "fargo_get_field_device(dens)");
  check(fargo_get_field_device(g_ctx, FARGO_FIELD_VRAD, Vrad_d), "fargo_get_field_device(vrad)");
  check(fargo_get_field_device(g_ctx, FARGO_FIELD_VTHETA, Vtheta_d), "fargo_get_field_device(vtheta)");
  check(fargo_get_field_device(g_ctx, FARGO_FIELD_TEMPERATURE, Temperature_d), "fargo_get_field_device(temp)");
  if (Adiabatic) check(fargo_get_field_device(g_ctx, FARGO_FIELD_ENERGY, Energy_d), "fargo_get_field_device(energy)");
  if (Cooling && Qplus_d) check(fargo_get_field_device(g_ctx, FARGO_FIELD_QPLUS, Qplus_d), "fargo_get_field_device(qplus)");
}

// the context's planets and run-time scalars into the reference's structures
void publish_state(PlanetarySystem *sys) {
  fargo_planet pl[64];
  int nb = 0;
  check(fargo_get_planets(g_ctx, pl, 64, &nb), "fargo_get_planets");
  for (int k = 0; k < nb && k < sys->nb; k++) {
    sys->x[k] = pl[k].x;
    sys->y[k] = pl[k].y;
    sys->vx[k] = pl[k].vx;
    sys->vy[k] = pl[k].vy;
    sys->mass[k] = pl[k].mass;
  }
  fargo_scalars s;
  check(fargo_get_scalars(g_ctx, &s), "fargo_get_scalars");
  PhysicalTime = s.physical_time;
  LostMass = s.lost_mass;
  OmegaFrame = s.omega_frame;
}
}  // namespace

// ReadVariables (src/Interpret.cu:100) wrapped at link time: the .par path, then the
// reference's own parser (its globals drive main()'s output cadence and dumps)
extern "C" void __real__Z13ReadVariablesPc(char *filename);
extern "C" void __wrap__Z13ReadVariablesPc(char *filename) {
  g_parfile = filename;
  __real__Z13ReadVariablesPc(filename);
}

// FillPolar1DArrays (src/SourceEuler.cu:66-162): creates the context and fills the
// host mesh arrays main()'s Cudamalloc copies; writes OUTPUTDIR/used_rad.dat.
void FillPolar1DArrays() {
  fargo_params p;
  fargo_params_default(&p);
  check(fargo_params_read(g_parfile.c_str(), &p), "fargo_params_read");
  std::string sw;
  if (SloppyCFL) sw += "c";
  if (CentrifugalBalance) sw += "b";
  if (!sw.empty()) check(fargo_params_apply_switches(sw.c_str(), &p), "fargo_params_apply_switches");
  fargo_planet pl[64];
  int nb = 0;
  if (p.planetconfig[0]) check(fargo_planets_read(p.planetconfig, &p, pl, 64, &nb), "fargo_planets_read");
  check(fargo_ctx_create(&p, pl, nb, FARGO_FP64, nullptr, &g_ctx), "fargo_ctx_create");
  const size_t n1 = (size_t)NRAD + 1;
  Radii = host_array(n1);
  Rinf = host_array(n1);
  Rmed = host_array(n1);
  Rsup = host_array(n1);
  Surf = host_array(n1);
  invRinf = host_array(n1);
  invSurf = host_array(n1);
  invRmed = host_array(n1);
  invdiffRsup = host_array(n1);
  invdiffRmed = host_array(n1);
  vt_cent = host_array(n1);
  powRmed = host_array(n1);
  check(fargo_get_mesh(g_ctx, Rinf, Rmed, Rsup, Surf), "fargo_get_mesh");
  // the reciprocal tables of src/SourceEuler.cu:127-150, from the same mesh
  for (int i = 0; i < NRAD; i++) {
    Radii[i] = Rinf[i];
    invRmed[i] = 1.0 / Rmed[i];
    invSurf[i] = 1.0 / Surf[i];
    invdiffRsup[i] = 1.0 / (Rsup[i] - Rinf[i]);
    invRinf[i] = 1.0 / Rinf[i];
    if (i > 0) invdiffRmed[i] = 1.0 / (Rmed[i] - Rmed[i - 1]);
    powRmed[i] = std::pow(Rmed[i], -2.5 + p.sigmaslope);
  }
  Radii[NRAD] = Rinf[NRAD];
  const std::string out = OUTPUTDIR + "used_rad.dat";
  FILE *f = std::fopen(out.c_str(), "w");
  if (!f) {
    std::printf("Can't write %s.\nProgram stopped.\n", out.c_str());
    std::exit(1);
  }
  for (int i = 0; i <= NRAD; i++) std::fprintf(f, "%.18g\n", Radii[i]);
  std::fclose(f);
}

// InitGasDensity / InitGasEnergy (src/Pframeforce.cu:31-52): the reference's 1D
// profiles (FillSigma / FillEnergy of Theo.o, which main() copies to the device),
// and the context's initial fields (the same profiles, and the .par's seeded noise)
void InitGasDensity(double *Dens) {
  FillSigma();
  check(fargo_get_field(g_ctx, FARGO_FIELD_DENS, Dens), "fargo_get_field(dens)");
}
void InitGasEnergy(double *Energy) {
  FillEnergy();
  check(fargo_get_field(g_ctx, FARGO_FIELD_ENERGY, Energy), "fargo_get_field(energy)");
}

// InitEuler (src/SourceEuler.cu:166-195): the host and device arrays the kept
// objects read, the initial velocities, and the fields on main()'s device arrays
void InitEuler(double *Vrad, double *Vtheta, double *Dens, double *Energy) {
  const size_t n = (size_t)size_grid;
  DensStar = host_array(n);
  DensInt = host_array(n);
  VradNew = host_array(n);
  VradInt = host_array(n);
  VthetaNew = host_array(n);
  VthetaInt = host_array(n);
  EnergyNew = host_array(n);
  EnergyInt = host_array(n);
  TemperInt = host_array(n);
  Potential = host_array(n);
  Pressure = host_array(n);
  SoundSpeed = host_array(n);
  Temperature = host_array(n);
  Qplus = host_array(n);
  DivergenceVelocity = host_array(n);
  Temperature_d = device_array(n);
  Energy_d = device_array(n);
  check(fargo_get_fields(g_ctx, nullptr, Vrad, Vtheta, nullptr, Temperature), "fargo_get_fields");
  (void)Dens;
  (void)Energy;
  publish_fields();
}

// AlgoGas (src/SourceEuler.cu:199-307): one DT on the library
void AlgoGas(Force *, double *, double *, double *, double *, double *, PlanetarySystem *sys, int) {
  int nsub = 0;
  check(fargo_step_DT(g_ctx, &nsub), "fargo_step_DT");
  publish_state(sys);
  publish_fields();
}

// compute_selfgravity (src/SgMain.cu:23-45) at set-up: the context computed it when
// it was created; Init_planetarysys_withSG (src/SgMain.cu:166-194): the planets'
// self-gravity-corrected initial speeds are the context's
void compute_selfgravity(double *, double, int, int) {}
void Init_planetarysys_withSG(PlanetarySystem *sys) { publish_state(sys); }

// AllocateForce / FreeForce (src/Force.cu:88-100): the force accumulator main() keeps
Force *AllocateForce(int dimfxy) {
  Force *f = (Force *)std::calloc(1, sizeof(Force));
  if (!f) fail("calloc", FARGO_ERR_INVALID);
  f->GlobalForce = host_array(4 * (size_t)dimfxy);
  return f;
}
void FreeForce(Force *force) {
  if (!force) return;
  std::free(force->GlobalForce);
  std::free(force);
}

// NearestPowerOf2 / IsPow2 (src/Kernels.cu:347-362), which size main()'s launch grids.
// The reference's IsPow2 evaluates x & ((x-1) == 0), true only for x == 1; main()
// then pads every size to the next power of two, and so does this one.
long NearestPowerOf2(long n) {
  if (!n) return n;
  long x = 1;
  while (x < n) x <<= 1;
  return x;
}
bool IsPow2(unsigned int x) { return x == 1u; }

// FViscosity (src/Viscosity.cu:33-50) for Theo.o's Qplusinit: the kinematic
// viscosity at r (constant, or alpha c_s^2 r^1.5 from the ring means of the sound
// speed held in GLOBAL_bufarray), with the cavity profile
double FViscosity(double r) {
  double nu = VISCOSITY;
  if (ViscosityAlpha) {
    int i = 0;
    while (i < NRAD - 1 && Rmed[i] < r) i++;
    nu = ALPHAVISCOSITY * GLOBAL_bufarray[i] * GLOBAL_bufarray[i] * std::pow(r, 1.5);
  }
  double rmin = CAVITYRADIUS - CAVITYWIDTH * ASPECTRATIO, rmax = CAVITYRADIUS + CAVITYWIDTH * ASPECTRATIO;
  const double scale = 1.0 + (PhysicalTime - PhysicalTimeInitial) * LAMBDADOUBLING;
  rmin *= scale;
  rmax *= scale;
  if (r < rmin) nu *= CAVITYRATIO;
  if (r >= rmin && r <= rmax) nu *= std::exp((rmax - r) / (rmax - rmin) * std::log(CAVITYRATIO));
  return nu;
}

// InitLabelKernel (launched by Init.o's InitLabel): 1 inside the planet's Hill
// sphere, 0 outside, cell centres at (Rmed_i cos phi_j, Rmed_i sin phi_j)
__global__ void InitLabelKernel(double *Label, double xp, double yp, double rhill, double *Rmed_dev, int nrad,
                                int nsec) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i >= nrad || j >= nsec) return;
  const double phi = (double)j / (double)nsec * 2.0 * PI;
  const double dx = Rmed_dev[i] * cos(phi) - xp, dy = Rmed_dev[i] * sin(phi) - yp;
  Label[(size_t)i * nsec + j] = sqrt(dx * dx + dy * dy) < rhill ? 1.0 : 0.0;
}

// MultiplyPolarGridbyConstantKernel (launched by LowTasks.o; main() leaves the call
// commented out): the density scaled, rings 0..nrad
__global__ void MultiplyPolarGridbyConstantKernel(double *Dens, int nrad, int nsec, double factor) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x, i = blockIdx.y * blockDim.y + threadIdx.y;
  if (i <= nrad && j < nsec) Dens[(size_t)i * nsec + j] *= factor;
}
