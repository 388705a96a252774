/*
 * fargo_gb300.h -- C-ABI of the GB300-native FARGO-ADSG 2D polar-grid hydro step.
 *
 * Every entry point is plain C: opaque context handle, plain pointers and sizes,
 * an int status (FARGO_OK == 0), never exit().  The reference exposes the same
 * operations as C++ host functions working on file-scope globals; each function
 * below names the reference interface it replaces (file:line in
 * MatiasFloresS/CudaProtoplanetaryDisks).
 *
 * Field layout (host and device): row-major [i*nsec + j], i = ring (radial, 0..nrad),
 * j = sector (azimuth, fastest).  Every field buffer holds (nrad+1)*nsec doubles;
 * ring nrad is the ghost ring of staggered radial quantities
 * (reference src/Main.cu:203 size_grid = (NRAD+1)*NSEC).
 */
#ifndef FARGO_GB300_H
#define FARGO_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------- */
#define FARGO_OK            0
#define FARGO_ERR_INVALID   1   /* bad argument or parameter set            */
#define FARGO_ERR_CUDA      2   /* CUDA runtime error (message in last_error) */
#define FARGO_ERR_IO        3   /* file could not be read or written        */
#define FARGO_ERR_NUMERIC   4   /* NaN/Inf in the CFL, CFL overflow, substep cap */
#define FARGO_ERR_STATE     5   /* call out of order (e.g. no context)      */

/* ---- precision modes ---------------------------------------------------- */
#define FARGO_FP64        0   /* every field and every operation in FP64 (parity mode) */
#define FARGO_FP32_BULK   1   /* fields, transport, source, viscosity in FP32; FP64 kept
                                 for planet RK5, force/indirect-term sums, azimuthal means,
                                 the FARGO mean/residual split and the SG convolution */

/* ---- per-substep entry points (fargo_substep 'which') ------------------- */
#define FARGO_SUB_BOUNDARY      1  /* ApplyBoundaryCondition   src/SideEuler.cu:31-41       */
#define FARGO_SUB_SOURCE        2  /* ComputePressureField + Substep1 + Substep2 + host +
                                      ActualiseGasVrad/Vtheta  src/SourceEuler.cu:278-284   */
#define FARGO_SUB_ENERGY        3  /* ComputeViscousTerms + Substep3 + ActualiseGasEnergy
                                      src/SourceEuler.cu:287-291                             */
#define FARGO_SUB_TRANSPORT     4  /* Transport                src/TransportEuler.cu:30-41  */
#define FARGO_SUB_TEMPERATURE   5  /* ComputeTemperatureField  src/SourceEuler.cu:484-489   */
#define FARGO_SUB_SOUNDSPEED    6  /* ComputeSoundSpeed        src/SourceEuler.cu:475-481   */
#define FARGO_SUB_POTENTIAL     7  /* ComputeAccel(star) + FillForcesArrays
                                      src/SourceEuler.cu:241-244                             */

/* ---- named fields for fargo_get_field ----------------------------------- */
#define FARGO_FIELD_DENS         0
#define FARGO_FIELD_VRAD         1
#define FARGO_FIELD_VTHETA       2
#define FARGO_FIELD_ENERGY       3
#define FARGO_FIELD_TEMPERATURE  4
#define FARGO_FIELD_PRESSURE     5
#define FARGO_FIELD_SOUNDSPEED   6
#define FARGO_FIELD_POTENTIAL    7
#define FARGO_FIELD_QPLUS        8
#define FARGO_FIELD_DIVERGENCE   9
#define FARGO_FIELD_SG_ACCR     10
#define FARGO_FIELD_SG_ACCT     11

/*
 * Parameter set: one member per global of include/Param.cuh:51-104 and the derived
 * flags of src/Interpret.cu:22-31 / src/Interpret.cu:130-206, plus the CLI switches of
 * src/Main.cu:115-179 that change the physics (-c, -b, -f).  The last block holds
 * extensions with no counterpart in the reference (seeded initial noise).
 */
typedef struct fargo_params {
  /* mesh */
  int    nrad, nsec;
  double rmin, rmax;
  int    log_grid;              /* RadialSpacing LOGARITHM */
  /* time */
  double dt;                    /* DT */
  int    ntot, ninterm;
  /* disk */
  double sigma0, sigmaslope, aspectratio, flaringindex;
  double viscosity, alphaviscosity;
  double imposeddiskdrift, eccentricity;
  double cavityradius, cavityratio, cavitywidth;
  double transitionradius, transitionratio, transitionwidth;
  double lambdadoubling;
  double adiabaticindex, coolingtime0;
  /* planets */
  double thicknesssmoothing, rochesmoothing;
  double masstaper;
  double releaseradius, releasedate;
  double omegaframe;
  /* derived flags (src/Interpret.cu:22-31) */
  int    fast_transport;        /* Transport != STANDARD            */
  int    open_inner;            /* InnerBoundary OPEN               */
  int    non_reflecting;        /* InnerBoundary NONREFLECTING      */
  int    evanescent;            /* InnerBoundary EVANESCENT         */
  int    is_disk;               /* Disk != NO                       */
  int    corotating;            /* Frame COROTATING / GUIDING-CENTER*/
  int    guiding_center;        /* Frame GUIDING-CENTER             */
  int    indirect_term;         /* IndirectTerm != NO               */
  int    exclude_hill;
  int    self_gravity, sg_zero_mode;
  int    adiabatic, cooling;
  int    cic_planet, forced_circular;
  int    viscosity_alpha;       /* AlphaViscosity != 0              */
  int    roche_smoothing;       /* RocheSmoothing != 0              */
  int    advect_label;
  int    outer_source_mass;
  int    write_density, write_velocity, write_energy;
  int    write_temperature, write_divv, write_qplus;
  /* CLI switches (src/Main.cu:115-179) */
  int    sloppy_cfl;            /* -c */
  int    centrifugal_balance;   /* -b */
  double scaling_factor;        /* -f */
  /* strings */
  char   outputdir[512];
  char   planetconfig[512];
  /* extensions (no counterpart in the reference): seeded uniform noise on the
     initial surface density / energy, Sigma *= 1 + amp*U[-1,1] (splitmix64) */
  double sigma_noise;
  double energy_noise;
  unsigned long long noise_seed;
} fargo_params;

/* One body of the planetary system (include/Types.cuh:2-12). */
typedef struct fargo_planet {
  double x, y, vx, vy, mass, acc;
  int    feel_disk, feel_others;
} fargo_planet;

/* Run-time scalars of the reference globals kept across steps. */
typedef struct fargo_scalars {
  double physical_time;         /* PhysicalTime  src/Viscosity.cu:21      */
  double omega_frame;           /* OmegaFrame    src/Main.cu:59           */
  double lost_mass;             /* LostMass      src/TransportEuler.cu:23 */
  double last_dt;               /* dt of the last hydro substep           */
  long long substeps;           /* hydro substeps done since creation     */
  int    last_cfl;              /* CFL integer of the last substep        */
  int    nb;                    /* number of planets                      */
  int    launches_per_substep;  /* kernels launched by one hydro substep  */
  int    launches_per_dt;       /* kernels launched once per DT (prefix)  */
  long long padded_substeps;    /* substeps run with dt = 0 to fill a loop body of two */
} fargo_scalars;

typedef struct fargo_ctx fargo_ctx;

/* ---- parameter interface ------------------------------------------------ */
/* Defaults of include/Param.cuh:51-104 and src/Interpret.cu:22-31. */
void fargo_params_default(fargo_params *p);
/* ReadVariables  src/Interpret.cu:100-212 (key/value .par file, '#' comments,
   case-folded keys).  Returns FARGO_ERR_IO when the file cannot be opened and
   FARGO_ERR_INVALID for the parameter conflicts the reference stops on
   (src/Interpret.cu:177-201). */
int  fargo_params_read(const char *parfile, fargo_params *p);
/* CLI switch string such as "-c" or "-bc" (src/Main.cu:115-151): sets sloppy_cfl /
   centrifugal_balance; returns FARGO_ERR_INVALID on characters the reference rejects. */
int  fargo_params_apply_switches(const char *sw, fargo_params *p);
/* InitPlanetarySystem  src/Psys.cu:168-217 (.cfg table: Name Distance Mass
   Accretion FeelsDisk FeelsOthers).  CICPlanet placement needs the mesh and is
   applied by fargo_ctx_create.  Writes at most cap bodies, *nb = bodies found. */
int  fargo_planets_read(const char *cfgfile, const fargo_params *p,
                        fargo_planet *out, int cap, int *nb);

/* ---- lifecycle ---------------------------------------------------------- */
/* Allocation + the initialisation sequence of main(), src/Main.cu:233-305:
   FillPolar1DArrays, InitGasDensity/InitGasEnergy (+ optional noise), the
   self-gravity set-up, Initialization (InitEuler, InitGasVelocities).
   stream: a cudaStream_t to launch on, or NULL for a context-owned stream. */
int  fargo_ctx_create(const fargo_params *p, const fargo_planet *planets, int nb,
                      int precision, void *stream, fargo_ctx **out);
/* Execution variants of a context: every combination gives bitwise the same
   results (the step's schedule changes, not its arithmetic), except az_chunks = 2
   and az_generic = 1, which sum the azimuthal ring mean in another order. */
typedef struct {
  int graph;       /* 1: one CUDA graph per DT, CFL loop on the device; 0: host loop */
  int pdl;         /* programmatic dependent launch between the step kernels */
  int pad;         /* two substeps per loop iteration, the second with dt = 0 after the DT's last */
  int sg_ahead;    /* the next substep's self-gravity ring transforms beside the end of this one */
  int rotate;      /* rotated DT loop (self-gravity of each substep launched by the previous one) */
  int az_generic;  /* barrier-per-phase azimuthal transport instead of the register-blocked one */
  int priority;    /* 0 equal stream priorities; 1 hydro chain above self-gravity; 2 the reverse */
  /* tile and launch shapes (each cell's arithmetic unchanged) */
  int cell_block;  /* CTA of the per-cell kernels: 0 64x4 sectors x rings, 1 32x8, 2 128x2, 3 256x1 */
  int rad_tma;     /* 1: radial transport on TMA-staged tiles in a persistent grid (when the rows
                      are 16-byte strided); 0: per-thread loads, one CTA per tile */
  int az_chunks;   /* four-cell chunks per thread of the register azimuthal sweep: 1 (one per
                      thread, up to the CTA size) or 2 (half the threads, two chunks each; the
                      ring mean is summed in another order, so results agree to rounding,
                      not bitwise) */
  int rad_col;     /* radial transport as a column march (one thread per sector walks a chunk
                      of rings with its stencil in registers; no shared memory, no barrier):
                      1 on, 0 off (rad_tma decides), -1 (default) on in FP32-bulk on grids
                      of at least 65536 sectors x ring chunks of 32 (off on smaller grids,
                      where it has too few threads, and in FP64, where it measured slower
                      than the TMA-staged tiles); FP32 results are bitwise those of the
                      tiles, FP64 agree to rounding */
} fargo_variant;
/* The default variant, with the FARGO_NO_GRAPH, FARGO_NO_PDL, FARGO_NO_PAD,
   FARGO_NO_SG_AHEAD, FARGO_ROTATE, FARGO_AZ_GENERIC and FARGO_PRIO switches
   applied (fargo_ctx_create uses it). */
void fargo_variant_default(fargo_variant *v);
/* fargo_ctx_create with an explicit variant (NULL: the default). */
int  fargo_ctx_create_variant(const fargo_params *p, const fargo_planet *planets, int nb, int precision,
                              void *stream, const fargo_variant *v, fargo_ctx **out);
void fargo_ctx_destroy(fargo_ctx *ctx);
/* Message of the last failing call on this context (never NULL). */
const char *fargo_last_error(const fargo_ctx *ctx);

/* ---- state -------------------------------------------------------------- */
/* DeviceToHostcudaMemcpy  src/Main.cu:605-616: copies (nrad+1)*nsec doubles per
   non-NULL buffer; temperature is the Temperature field of the last substep. */
int  fargo_get_fields(fargo_ctx *ctx, double *dens, double *vrad, double *vtheta,
                      double *energy, double *temperature);
/* Overwrites the state fields (host -> device); NULL leaves a field unchanged. */
int  fargo_set_fields(fargo_ctx *ctx, const double *dens, const double *vrad,
                      const double *vtheta, const double *energy);
/* One named field (FARGO_FIELD_*), (nrad+1)*nsec doubles. */
int  fargo_get_field(fargo_ctx *ctx, int which, double *host);
/* The same field copied device to device into the caller's FP64 array dev
   ((nrad+1)*nsec doubles, the reference's layout; FP32-bulk fields widened), on the
   context's stream, then synchronised.  For a host driver that keeps device arrays
   of its own: the reference's DeviceToHostcudaMemcpy (src/Main.cu:605-616) reads
   Dens_d, Vrad_d, Vtheta_d, Energy_d, Temperature_d, Qplus_d.  Fields held on the
   host or completed there (isothermal sound speed, potential): FARGO_ERR_INVALID. */
int  fargo_get_field_device(fargo_ctx *ctx, int which, double *dev);
int  fargo_get_planets(fargo_ctx *ctx, fargo_planet *out, int cap, int *nb);
int  fargo_get_scalars(fargo_ctx *ctx, fargo_scalars *s);
/* 1D mesh arrays (FillPolar1DArrays src/SourceEuler.cu:66-162): Rinf, Rmed, Rsup,
   Surf, each nrad+1 doubles (any may be NULL). */
int  fargo_get_mesh(fargo_ctx *ctx, double *rinf, double *rmed, double *rsup, double *surf);

/* ---- stepping ----------------------------------------------------------- */
/* AlgoGas  src/SourceEuler.cu:199-307 (include/SourceEuler.cuh:10-11): one DT,
   CFL-subcycled.  *nsub (may be NULL) = hydro substeps taken.  Synchronous. */
int  fargo_step_DT(fargo_ctx *ctx, int *nsub);
/* ndt consecutive AlgoGas calls, launched back to back (no host sync inside);
   the main loop of src/Main.cu:309-333 without its output branch. */
int  fargo_run(fargo_ctx *ctx, int ndt, long long *nsub);
/* Asynchronous variant: enqueues ndt DT-steps on the context stream and returns. */
int  fargo_run_async(fargo_ctx *ctx, int ndt);
int  fargo_sync(fargo_ctx *ctx);
/* One hydro substep of length dt (the body of the AlgoGas while loop,
   src/SourceEuler.cu:223-302) with the CFL evaluation skipped. */
int  fargo_substep_full(fargo_ctx *ctx, double dt);
/* Per-substep entry points for parity harnesses (FARGO_SUB_*):
   ApplyBoundaryCondition (include/SideEuler.cuh:1), Substep1/2/host
   (include/SourceEuler.cuh:12-20), Substep3, Transport (include/TransportEuler.cuh:1),
   ComputeTemperatureField, ComputeSoundSpeed, ComputeAccel + FillForcesArrays
   (include/SideEuler.cuh:10, include/Pframeforce.cuh:4). */
int  fargo_substep(fargo_ctx *ctx, int which, double dt);
/* ConditionCFL  src/SourceEuler.cu:520-546 (include/SourceEuler.cuh:20). */
int  fargo_condition_cfl(fargo_ctx *ctx, double deltaT, int *cfl);

/* ---- output (src/Output.cu) ---------------------------------------------- */
/* SendOutput + WritePlanetSystemFile  src/Output.cu:133-181 / 76-131:
   OUTPUTDIR/<name>/<name><index>.dat raw FP64 nrad*nsec, names dens, vrad,
   vtheta, energy, temperature, divergence, qplus; planet<k>.dat rows. */
int  fargo_write_outputs(fargo_ctx *ctx, int index);
/* WriteDim (src/Output.cu:19-35) + EmptyPlanetSystemFile (37-58). */
int  fargo_write_dims(fargo_ctx *ctx);
/* Restart from output `index` of an earlier run with the same parameters and
   OUTPUTDIR: FARGO's "-s index", which the reference parses but never acts on
   (src/Main.cu:152-160).  Density, velocities (and energy when adiabatic) from
   the field dumps (ring nrad keeps the created context's values: the dumps hold
   nrad rings); positions, velocities and masses of the planets, PhysicalTime,
   OmegaFrame and LostMass from row `index` of planet<k>.dat; the planet files
   are cut to the rows before `index`, so that writing output `index` again
   continues them.  The run's start time stays that of the created context.
   FARGO_ERR_IO when a file or row is missing; without planets the time is
   index * NINTERM * DT. */
int  fargo_restart(fargo_ctx *ctx, int index);

/* ---- disk forces and the torque logs --------------------------------------- */
#define FARGO_FORCE_LEVELS 11   /* dimfxy, src/Main.cu:74 */
/* ComputeForce (src/Force.cu:102-131, ComputeForceKernel src/Kernels.cu:693-729):
   the disk's force on the point (x, y) with the given smoothing, split into inner
   (Rmed < a) and outer cells and over FARGO_FORCE_LEVELS Hill cuts (level k
   weights a cell by 1 - exp(-d^2 / (rh k / (levels - 1))^2); level 0 is uncut).
   global_force: 4 * FARGO_FORCE_LEVELS doubles, fx inner [k], fx outer
   [levels + k], fy inner [2 levels + k], fy outer [3 levels + k] (the reference's
   GlobalForce).  mass is unused, as in the reference.  Synchronous. */
int  fargo_compute_force(fargo_ctx *ctx, double x, double y, double smoothing, double mass, double a, double rh,
                         double *global_force);
/* UpdateLog (src/Force.cu:19-84; the reference's call is commented out at
   src/Main.cu:315): for every planet k, appends to OUTPUTDIR/tqwk<k>.dat the row
   timestep, the torques of the inner, outer, Hill-cut inner and Hill-cut outer
   disk, the same four powers, PhysicalTime; without self-gravity also, per
   level l, to tqwk<k>_<l>.dat: timestep, inner and outer torque, inner and
   outer power, PhysicalTime.  Synchronous. */
int  fargo_update_log(fargo_ctx *ctx, int timestep);

/* ---- measurement (no counterpart in the reference) ----------------------- */
/* Runs reps hydro substeps launch by launch with a CUDA event after every kernel
   and returns the mean device time (ms) of each kernel of one substep, in launch
   order; *nkernels = kernels per substep.  Advances the state like reps substeps. */
int  fargo_time_substep_kernels(fargo_ctx *ctx, int reps, double *ms_per_kernel, int cap, int *nkernels);
/* Name of kernel k of the last fargo_time_substep_kernels call (NULL if none). */
const char *fargo_substep_kernel_name(const fargo_ctx *ctx, int k);
/* Measured peak of the FP64 pipe of the current device: thread-level FP64 fused
   multiply-adds per second (*dfma_per_s) of a kernel of independent DFMA chains
   filling every SM, timed with CUDA events after a warm-up launch.  The roofline
   of the FP64 mode, whose kernels are bound by this pipe.  Synchronous. */
int  fargo_fp64_pipe_peak(double *dfma_per_s);
/* Self-test of the FP64 step's two divides on the device: q_step[k] = a[k] / b[k]
   as the per-cell arithmetic divides (the reciprocal estimate, one Newton step,
   the quotient and one correction: the correctly rounded quotient except within
   about 2^-80 of a rounding midpoint) and q_lim[k] as the slope limiters divide
   (without the correction: relative error about 2^-40); both IEEE a / b outside
   |a|, |b| in [2^-500, 2^501).  n in 1..2^24.  Synchronous. */
int  fargo_div_selftest(const double *a, const double *b, int n, double *q_step, double *q_lim);
/* Self-test of the 5th-generation tensor-core path (tcgen05, sm_100 family): one
   CTA computes d (128 x n, FP32, row-major) = a (128 x k, BF16 bit patterns,
   row-major) x b (n x k, BF16, row-major)^T with k / 16 MMAs accumulating in
   tensor memory, read back with tcgen05.ld.  n in 16..256 and k in 16..128,
   multiples of 16.  The operands are staged in the no-swizzle K-major layout with
   the core matrices adjacent along K packed together (mode 0) or those adjacent
   along the rows (mode 1); mode 2 stages as mode 0 but swaps the two stride fields
   of the descriptors (the other reading of the descriptor; its product is not
   expected to be the matrix product).  Synchronous; FARGO_ERR_NUMERIC if an MMA did
   not complete within its bounded wait. */
int  fargo_tc_selftest(const unsigned short *a, const unsigned short *b, int n, int k, int mode, float *d);

/* ---- allocation-free CFL (no counterpart in the reference) --------------- */
/* The CFL integer of ConditionCFL for callers that cannot call cudaMalloc
   (device memory owned by another allocator, or a loop that must not take
   cudaMalloc's implicit synchronisation).  Inputs are the caller's FP64 device
   arrays: vrad, vtheta, soundspeed ((nrad+1)*nsec each, ring-major) and rinf,
   rmed, rsup (nrad+1 each); *cfl_out is a device int written on `stream`
   (-1 when the time step is not finite).  Arithmetic: the reference's own
   (ring means summed in sector order, every term divided as written, no fused
   multiply-add), so on identical inputs the integer is the reference's;
   fargo_condition_cfl (tree sums, per-ring reciprocals) can differ from it by one
   at a rounding tie.  Allocates nothing: its scratch is a fixed array inside the
   library, at most 16384 rings and 16384 sectors (larger: FARGO_ERR_INVALID).
   The first call on a device sets up that device (make it before any stream
   capture, and do not use the entry point across a device reset); calls that
   overlap on the GPU race on the array. */
int  fargo_condition_cfl_noalloc(const double *vrad, const double *vtheta, const double *soundspeed,
                                 const double *rinf, const double *rmed, const double *rsup,
                                 int nrad, int nsec, int fast_transport, double deltaT,
                                 void *stream, int *cfl_out);

/* ---- ensembles (no counterpart in the reference) -------------------------- */
/* n independent disks (the batched-ensemble workload): disk k has params[k] and
   the nplanets[k] bodies that follow those of disks 0..k-1 in planets.  Each disk
   is a context of its own (own fields, DT graph, CFL step and streams); the batch
   enqueues the disks' DT graphs round-robin so that the GPU runs many disks at
   once.  A disk's results are bitwise those of the same disk run alone. */
typedef struct fargo_batch fargo_batch;
int  fargo_batch_create(int n, const fargo_params *params, const fargo_planet *planets, const int *nplanets,
                        int precision, fargo_batch **out);
/* The same with every disk in variant v (NULL: the default). */
int  fargo_batch_create_variant(int n, const fargo_params *params, const fargo_planet *planets,
                                const int *nplanets, int precision, const fargo_variant *v, fargo_batch **out);
/* Fused execution of the batch: from this call on, fargo_batch_run_async
   advances every disk by launching each substep kernel once per lane of disks
   instead of running one graph per disk -- one CUDA graph per DT round: every
   disk's DT start, then a conditional while loop whose body is one substep of
   every disk whose DT is not yet over (masked subcycling: each disk keeps its own
   CFL step, substep count and DT; finished disks' blocks return at once).
   fargo_batch_fuse gathers the disks of each ring width into a lane (one launch
   per kernel per width, the lanes side by side in the loop body, every block
   shaped for its width); fargo_batch_fuse_by_width(b, 0) puts every disk in one
   lane (one launch per kernel for the whole ensemble, blocks shaped for the
   widest ring).  Bitwise the results of the disks run alone.
   FARGO_ERR_INVALID (reason in fargo_batch_last_error) when a disk uses
   self-gravity, an open, non-reflecting or evanescent boundary, the sloppy CFL
   or a ring too wide for the register azimuthal sweep. */
int  fargo_batch_fuse(fargo_batch *b);
int  fargo_batch_fuse_by_width(fargo_batch *b, int by_width);
/* The reason of the last failed fargo_batch_fuse ("" if none). */
const char *fargo_batch_last_error(const fargo_batch *b);
/* Kernel launches of the fused form: per substep (all disks) and per DT round. */
int  fargo_batch_fused_launches(const fargo_batch *b, int *per_substep, int *per_dt);
/* Lanes of the fused form. */
int  fargo_batch_fused_lanes(const fargo_batch *b, int *lanes);
/* Starts a DT round of the fused form, then runs reps substeps of it launch by
   launch (lanes one after another, a CUDA event after every launch) and returns
   the mean device time (ms) of each launch group of one substep, in launch order;
   *ngroups = groups per substep.  Advances the disks like reps substeps of a
   round (a disk whose DT ends sooner stops there). */
int  fargo_batch_fused_time_kernels(fargo_batch *b, int reps, double *ms_per_group, int cap, int *ngroups);
/* Kernel of group k of the last fargo_batch_fused_time_kernels call (NULL if none). */
const char *fargo_batch_fused_kernel_name(const fargo_batch *b, int k);
/* Autotuner of the ensemble's schedule: starting from the default variant, tries
   the alternatives of one knob at a time (padding, stream priorities, the
   self-gravity schedule when a disk has self-gravity, programmatic launch), each
   on a fresh batch of these disks (one warm-up DT, then ndt DTs on every disk,
   host clock around enqueue and synchronisation), and keeps an alternative that
   raises the batch's cell-updates/s by more than 0.5%.  *best: the variant kept;
   *rate_best, *rate_default (may be NULL): its rate and the default's.  The
   variants give identical results, so the choice changes speed only. */
int  fargo_batch_autotune(int n, const fargo_params *params, const fargo_planet *planets, const int *nplanets,
                          int precision, int ndt, fargo_variant *best, double *rate_best, double *rate_default);
void fargo_batch_destroy(fargo_batch *b);
int  fargo_batch_size(const fargo_batch *b);
/* Context of disk k (owned by the batch), for fields, planets and scalars. */
fargo_ctx *fargo_batch_disk(fargo_batch *b, int k);
/* ndt DTs on every disk, enqueued without a host synchronisation. */
int  fargo_batch_run_async(fargo_batch *b, int ndt);
int  fargo_batch_sync(fargo_batch *b);
/* Every disk advances whole DTs of its own until its physical time reaches t_end;
   *nsub (may be NULL) = substeps of all disks.  On a device error the status is
   that disk's and *failed (may be NULL) = its index, else -1. */
int  fargo_batch_advance(fargo_batch *b, double t_end, long long *nsub, int *failed);

/* ---- learned coarse-grid correction (no counterpart in the reference) ---- */
/* The stencil MLP: 128 inputs -> 64 (GELU) -> 64 (GELU) -> 2 outputs, BF16 on
   the tensor cores with FP32 accumulation.  Parameters: FP32 blob of
   FARGO_MLP_NPARAM floats, W1 [128][64], b1 [64], W2 [64][64], b2 [64], W3 [64][8]
   (columns 2..7 zero), b3 [8] (entries 2..7 zero); W[in][out].  GELU in its tanh
   form.  Inputs: BF16 [n][128] device rows, 16-byte aligned; outputs and their
   gradients: FP32 [n][2] device rows, 8-byte aligned. */
#define FARGO_MLP_NPARAM (128 * 64 + 64 + 64 * 64 + 64 + 64 * 8 + 8)
typedef struct fargo_mlp fargo_mlp;
/* Calls of at most max_rows rows; the workspace is the per-CTA gradient partials
   of one persistent grid (the device's resident CTAs). */
int  fargo_mlp_create(int max_rows, fargo_mlp **out);
void fargo_mlp_destroy(fargo_mlp *m);
/* Host FP32 blobs; setting the parameters resets the Adam moments. */
int  fargo_mlp_set_params(fargo_mlp *m, const float *host);
int  fargo_mlp_get_params(fargo_mlp *m, float *host);
/* Gradient of the last fargo_mlp_backward (host FP32 blob). */
int  fargo_mlp_get_grad(fargo_mlp *m, float *host);
/* y = f(x) on n rows.  train is accepted for compatibility and ignored: the
   backward pass recomputes the forward pass of its rows. */
int  fargo_mlp_forward(fargo_mlp *m, const void *x_bf16, int n, float *y, int train, void *stream);
/* The forward pass's tensor-core path: FARGO_MLP_MMA_SYNC (default: 16-row warp
   tiles, mma.sync m16n8k16, every activation in registers) or FARGO_MLP_TCGEN05
   (128-row tiles, tcgen05.mma with the accumulators in tensor memory, each hidden
   layer's GELU epilogue through shared memory).  Their outputs are bitwise equal on
   GB300; the mma.sync path measured faster (31.8 against 41.1 us on 196,608 rows:
   the GELU epilogue, not the tensor pipe, bounds both). */
#define FARGO_MLP_TCGEN05 0
#define FARGO_MLP_MMA_SYNC 1
int  fargo_mlp_set_tensor_path(fargo_mlp *m, int path);
/* FARGO_ERR_NUMERIC if an MMA of a tcgen05 forward pass did not complete within
   its bounded wait (the pass then leaves its rows unwritten).  Synchronous. */
int  fargo_mlp_status(fargo_mlp *m);
/* dL/dparameters from dL/dy (FP32 [n][2]) of the rows x; summed over the rows in
   a fixed order (deterministic on a given device). */
int  fargo_mlp_backward(fargo_mlp *m, const void *x_bf16, int n, const float *dy, void *stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) with learning rate lr. */
int  fargo_mlp_adam(fargo_mlp *m, float lr, void *stream);

/* Coupling of the MLP to a coarse disk (device buffers; fields of esize bytes,
   (nrad+1)*nsec elements; rmed and surf: FP64 device arrays of nrad+1).
   features: x (BF16 [nrad*nsec][128]) from density and velocities; norm: 125 means
   then 125 deviations of the inputs.  divergence: the density correction
   ds (FP32 [nrad*nsec]) of the network outputs y (FP32 [nrad*nsec][2]) scaled by
   scale (mass conserved by construction).  loss: ds, e = dL/dds, dy = dL/dy and
   *loss (device double) = sum (ds - target)^2, for L = that sum * inv_var / n
   (part: (n + 255) / 256 doubles of scratch). */
int  fargo_learned_features(int esize, const void *dens, const void *vrad, const void *vtheta, const double *rmed,
                            int nrad, int nsec, double phi_planet, const float *norm, void *x_bf16, void *stream);
int  fargo_learned_divergence(const float *y, const double *surf, int nrad, int nsec, float scale, float *ds,
                              void *stream);
/* Ring-neutral outputs: subtracts from the radial outputs y[.][0] of every ring
   their mean over the ring, in place.  Applied to y before fargo_learned_divergence,
   the correction leaves every ring's mass (the azimuthally averaged density)
   unchanged; applied to dL/dy after fargo_learned_loss, it gives the gradient
   through the projection (the projection is its own adjoint). */
int  fargo_learned_ring_center(float *y, int nrad, int nsec, void *stream);
/* fargo_learned_divergence on the disk's grid with a positivity limiter
   (donor-cell, as in flux-corrected transport): every face flux of the
   correction is scaled by the fraction of its outflows its donor cell can
   afford, so that no cell loses more than beta (0 < beta < 1) of its current
   mass; each face keeps one flux, so the total mass is conserved as without the
   limiter.  Where the corrections are small against the density nothing
   changes.  Runs on the context's stream: y must be complete when it is
   called.  Synchronous. */
int  fargo_learned_divergence_limited(fargo_ctx *ctx, const float *y, float scale, float beta, float *ds);
int  fargo_learned_loss(const float *y, const float *target, const double *surf, int nrad, int nsec, float scale,
                        float inv_var, float *ds, float *e, float *dy, double *part, double *loss, void *stream);
/* The coarse disk's density and velocities := the restriction of the fine disk's
   (fine grid = factor x coarse in both directions; area-weighted density,
   interface velocities averaged).  Synchronous. */
int  fargo_learned_restrict(fargo_ctx *fine, fargo_ctx *coarse, int factor);
/* Adds ds (device FP32 [nrad*nsec]) to the disk's density when every cell stays
   positive and finite and |sum ds Surf| <= 1e-5 sum |ds Surf| (the plain step
   judges the correction); *accepted = 1 then, else 0 and nothing changes.
   *dmass (may be NULL) = sum ds Surf.  Synchronous. */
int  fargo_learned_apply(fargo_ctx *ctx, const float *ds, int *accepted, double *dmass);
/* fargo_learned_features on the disk's own state (the first planet's azimuth);
   and the disk's density (rings 0..nrad-1) as FP32 into a device buffer.  Synchronous. */
int  fargo_learned_features_ctx(fargo_ctx *ctx, const float *norm, void *x_bf16);
int  fargo_learned_density(fargo_ctx *ctx, float *out);

#ifdef __cplusplus
}
#endif
#endif /* FARGO_GB300_H */
