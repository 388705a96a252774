// fargo_internal.h -- host-side definitions shared by the library's translation units.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "fargo_gb300.h"
#include "fargo_physics.h"

// Per-ring table rows: RT_COUNT values per ring for rings 0..nrad, stored ring after
// ring (the rows of one ring adjacent).
enum RingTab {
  RT_RINF = 0, RT_RMED, RT_RSUP, RT_SURF, RT_INVRINF, RT_INVSURF, RT_INVRMED,
  RT_INVDIFFRSUP, RT_INVDIFFRMED,
  RT_DXTHETA,      // 2.0*PI/(double)nsec*Rmed[i]       (Substep1Kernel, kernel, StarTheta)
  RT_INVDXTHETA,   // 1.0/RT_DXTHETA
  RT_DXTHETA_CFL,  // Rmed[i]*2.0*PI/(double)nsec       (ConditionCFLKernel2D1)
  RT_SUPPTORQUE,   // IMPOSEDDISKDRIFT*0.5*pow(Rmed,-2.5+SIGMASLOPE)
  RT_CS,           // isothermal sound speed of the ring
  RT_NU,           // viscosity_array
  RT_DRAD,         // Rsup - Rinf
  RT_SIGMAMED, RT_ENERGYMED, RT_COOLTIME, RT_QPLUSMED,
  RT_SGSQRT,       // sqrt(Rmed/Rmed0)
  RT_SGRATIO,      // Rmed/Rmed0
  RT_CSMEAN,       // ring mean of SoundSpeed (GLOBAL_bufarray)
  RT_SGNORMR,      // normaccr of ComputeSgAccKernel (src/Kernels.cu:902-905)
  RT_SGNORMT,      // normacct
  RT_INVDRAD,      // 1/(Rsup - Rinf)
  RT_INVDXTHETA_CFL,  // 1/RT_DXTHETA_CFL
  RT_INVMIND,      // 1/min(Rsup - Rinf, RT_DXTHETA_CFL)
  RT_VKEP2,        // squared sub-Keplerian edge speed before the self-gravity term (t = t0)
  RT_R15,          // pow(Rmed, 1.5) of the alpha viscosity
  RT_CAVFAC,       // cavity factor of FViscosity (t = t0)
  RT_AZSHIFT,      // nsec/(2 pi Rmed): the FARGO shift per unit (Vtheta mean x dt)
  RT_INVSIGMAMED,  // 1/SigmaMed (0 where SigmaMed is 0)
  RT_COUNT
};

// FP64 staging slots (one field each) of a context's FP32 host <-> device transfers
#define FARGO_STAGING_SLOTS 5

struct HostState {
  int nrad = 0, nsec = 0;
  size_t size_grid = 0;
  std::vector<double> Radii, Rinf, Rmed, Rsup, Surf, invRinf, invSurf, invRmed, invdiffRsup, invdiffRmed;
  std::vector<double> SigmaMed, SigmaInf, EnergyMed, CoolingTimeMed, QplusMed, nu, cs_mean;
  std::vector<double> Dens, Vrad, Vtheta, Energy, SoundSpeed, Pressure, Temperature;
  std::vector<double> cosF, sinF, cosP, sinP;   // force and potential angle tables
  std::vector<double> Kr, Kt;                   // self-gravity kernels, 2*nrad x nsec
  double OmegaFrame = 0.0;
};

// setup.cpp
void host_fill_mesh(const fargo_params &p, HostState &h);
void host_init_density_energy(const fargo_params &p, HostState &h);
void host_init_planets(const fargo_params &p, const HostState &h, const fargo_planet *pl, int nb, Ctl &c);
void host_sg_kernel(const fargo_params &p, HostState &h, DevParams &dp);
void host_init_planets_sg(const fargo_params &p, const HostState &h, const std::vector<double> &axi_accr, Ctl &c);
void host_init_euler(const fargo_params &p, HostState &h, const DevParams &dp, Ctl &c);
void host_ring_table(const fargo_params &p, const HostState &h, const DevParams &dp, std::vector<double> &tab);
DevParams host_dev_params(const fargo_params &p, int nb);
long fargo_nearest_pow2(long n);

// Device view of a context for the kernels outside the step (the learned
// correction, fargo_learned.cu; the disk-force diagnostic, fargo_force_diag.cu);
// the call reads the control block (synchronises the context's stream)
struct DiskView {
  void *dens, *vrad, *vtheta;   // fields, (nrad + 1) * nsec elements of esize bytes
  int esize, nrad, nsec;
  void *stream;                 // the context's cudaStream_t
  const double *rmed, *surf;    // host mesh, nrad + 1 each
  double planet_phi;            // azimuth of the first planet (0 without one)
  // device copies of rmed and surf, and scratch (a candidate density, 3 doubles
  // per ring), allocated with the context on first use
  const double *rmed_dev, *surf_dev;
  double *ring;
  void *cand;
};
extern "C" int fargo_disk_view(fargo_ctx *c, DiskView *v);

// output.cpp
int host_write_field(const std::string &outdir, const char *name, int index, const double *data, size_t n);
int host_write_planet_row(const std::string &outdir, int k, int index, const fargo_planet &b, double lost_mass,
                          double physical_time, double omega_frame);
int host_write_dims(const fargo_params &p, int nb);
int host_write_used_rad(const fargo_params &p, const HostState &h);
int host_read_field(const std::string &outdir, const char *name, int index, double *data, size_t n);
int host_read_planet_row(const std::string &outdir, int k, int index, fargo_planet &b, double *lost_mass,
                         double *physical_time, double *omega_frame);
int host_truncate_planet_file(const std::string &outdir, int k, int index);
int host_append_row(const std::string &outdir, const std::string &file, int index, const double *v, int nv);

// Fused execution of an ensemble (fargo_ctx.cu): one launch of each substep kernel
// for all disks, one CUDA graph per DT round (the DT start of every disk, then a
// conditional while loop of substeps that runs until the last disk's DT is done).
struct fargo_fused;
int fused_create(fargo_ctx *const *disks, int n, int by_width, fargo_fused **out, std::string *why);
int fused_run(fargo_fused *f, int ndt);
int fused_sync(fargo_fused *f);
void fused_destroy(fargo_fused *f);
int fused_launches(const fargo_fused *f, int *per_substep, int *per_dt);
int fused_lanes(const fargo_fused *f);
int fused_time_kernels(fargo_fused *f, int reps, double *ms, int cap, int *ngroups);
const char *fused_kernel_name(const fargo_fused *f, int k);
