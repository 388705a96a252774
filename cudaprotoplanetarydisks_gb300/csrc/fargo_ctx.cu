// fargo_ctx.cu -- disk context, device memory, graph of one DT, and the C-ABI.
//
// A context owns every device buffer of one disk (the reference keeps them in
// file-scope globals allocated by Cudamalloc, src/Main.cu:660-827, and friends).
// One DT (AlgoGas, src/SourceEuler.cu:199-307) is one CUDA graph: a prefix
// (DT start, sound speed of the energy equation) followed by a conditional WHILE
// node whose body is one hydro substep; the substep's last kernel sets the loop
// condition from the device-side dtemp, so a DT runs without any host sync.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "fargo_device.cuh"
#include "fargo_internal.h"
#include "fargo_kernels.cuh"

struct fargo_ctx {
  fargo_params P;
  DevParams dp;
  int precision = FARGO_FP64;
  int nb = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  SideBranch side = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // side streams of a substep
  HostState h;
  std::string err = "no error";
  Ctl *d_ctl = nullptr;
  Ctl *pin_ctl = nullptr;
  std::vector<void *> allocs;
  size_t esize = 8;
  // fields (element type T = double or float)
  void *dens = nullptr, *vrad = nullptr, *vtheta = nullptr, *energy = nullptr, *cs = nullptr;
  void *pressure = nullptr, *temperature = nullptr, *potential = nullptr;
  void *vradint = nullptr, *vthetaint = nullptr, *energyint = nullptr;
  void *qplus = nullptr, *divv = nullptr, *taurr = nullptr, *taurp = nullptr, *taupp = nullptr;
  void *densr = nullptr, *energyr = nullptr, *radmomp = nullptr, *radmomm = nullptr;
  void *thetamomp = nullptr, *thetamomm = nullptr, *sg_accr = nullptr, *sg_acct = nullptr;
  void *az_scratch = nullptr, *rt = nullptr, *nu = nullptr, *cosP = nullptr, *sinP = nullptr;
  void *rdsum = nullptr;
  void *cosFt = nullptr, *sinFt = nullptr;
  double *rt64 = nullptr, *csmean = nullptr, *cosF = nullptr, *sinF = nullptr;
  double *ring_force = nullptr, *lostbydisk = nullptr;
  // self-gravity
  void *spec2_r = nullptr, *spec2_t = nullptr;
  void *spec_r = nullptr, *spec_t = nullptr, *khat_r = nullptr, *khat_t = nullptr, *tw1 = nullptr, *tw0 = nullptr;
  double2 *khat64_r = nullptr, *khat64_t = nullptr, *tw1_64 = nullptr, *tw0_64 = nullptr;  // FP64 set-up
  double *kr = nullptr, *kt = nullptr;
  int rad1[16], nst1 = 0, rad0[16], nst0 = 0;
  size_t az_smem = 0;
  int az_regs = 0;
  double *staging = nullptr;   // FP64 staging slots of host <-> device transfers (FP32 fields)
  double *lx_rmed = nullptr, *lx_surf = nullptr, *lx_ring = nullptr;  // learned correction (first use)
  void *lx_cand = nullptr;
  int launches_per_substep = 0, launches_per_dt = 0;
  std::vector<std::string> kernel_names;
  // graph of one DT
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  unsigned long long cond_handle = 0;
  bool use_graph = true;
  bool use_pdl = true;   // programmatic dependent launch between the step kernels
  bool use_rotation = false;  // rotated DT loop (self-gravity ahead of each substep)
  bool use_sg_ahead = true;   // ring transforms of the next substep beside the end of this one
  bool use_pad = true;        // two substeps per loop body, the second padded (dt = 0) after the DT's last
  bool sg_generic = false;    // run-time FFT plans only (the compile-time ones compared in the tests)
  bool az_generic = false;    // barrier-per-phase azimuthal kernel instead of the register-blocked one
  // radial transport with TMA-staged tiles (k_transport_radial_tma): its tensor maps
  // and persistent grid; off when the rows are not 16-byte strided or FARGO_NO_TMA=1
  RadMaps rad_maps;
  bool use_tma = false;
  int rad_grid = 0;
  bool want_tma = true;       // the variant asks for the TMA radial transport
  int cell_block = 0;         // per-cell kernels' CTA shape (fargo_variant.cell_block)
  int az_chunks = 1;          // chunks per thread of the register azimuthal sweep
  bool rad_col = false;       // column-march radial transport
};

namespace {
// ring buffers of the barrier-per-phase azimuthal kernel (AZ_NARR in fargo_kernels.cu)
constexpr int AZ_NARR_HOST = 12;

// 2D tensor maps (sectors x rings 0..nrad, one box = RAD_BW sectors x RAD_BR rings,
// zero fill outside) of the density, Vrad, Vtheta and (energy equation) energy,
// for k_transport_radial_tma.  TMA needs 16-byte row strides (nsec * element size).
// The encoder is the driver's cuTensorMapEncodeTiled, reached through the runtime.
template <class T>
void make_rad_maps(fargo_ctx *c) {
  c->use_tma = false;
  const size_t E = sizeof(T);
  if (((size_t)c->P.nsec * E) % 16 != 0) return;
  PFN_cuTensorMapEncodeTiled_v12000 enc = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", (void **)&enc, 12000, cudaEnableDefault, &q) !=
          cudaSuccess ||
      q != cudaDriverEntryPointSuccess || !enc)
    return;
  const cuuint64_t dims[2] = {(cuuint64_t)c->P.nsec, (cuuint64_t)c->P.nrad + 1};
  const cuuint64_t strides[1] = {(cuuint64_t)c->P.nsec * E};
  const cuuint32_t box[2] = {(cuuint32_t)RAD_BW(T), (cuuint32_t)RAD_BR};
  const cuuint32_t es[2] = {1, 1};
  const CUtensorMapDataType dt = E == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  void *src[4] = {c->dens, c->vrad, c->vtheta, c->P.adiabatic ? c->energy : c->dens};
  CUtensorMap *dst[4] = {&c->rad_maps.dens, &c->rad_maps.vrad, &c->rad_maps.vtheta, &c->rad_maps.energy};
  for (int f = 0; f < 4; f++) {
    if (!src[f]) return;
    if (enc(dst[f], dt, 2, src[f], dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
      return;
  }
  c->rad_grid = rad_tma_grid<T>(c->P.nrad, c->P.nsec);
  c->use_tma = c->rad_grid > 0;
}

int set_err(fargo_ctx *c, int code, const std::string &msg) {
  if (c) c->err = msg;
  return code;
}

#define CK(call)                                                                                      \
  do {                                                                                                \
    cudaError_t e_ = (call);                                                                          \
    if (e_ != cudaSuccess)                                                                            \
      return set_err(c, FARGO_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));         \
  } while (0)

template <class T>
KArgs<T> make_args(const fargo_ctx *c) {
  KArgs<T> a;
  std::memset(&a, 0, sizeof(a));
  a.P = c->dp;
  DiskPtrs<T> &d = a.d;
  d.dens = (T *)c->dens;
  d.vrad = (T *)c->vrad;
  d.vtheta = (T *)c->vtheta;
  d.energy = (T *)c->energy;
  d.cs = (T *)c->cs;
  d.pressure = (T *)c->pressure;
  d.temperature = (T *)c->temperature;
  d.potential = (T *)c->potential;
  d.vradint = (T *)c->vradint;
  d.vthetaint = (T *)c->vthetaint;
  d.energyint = (T *)c->energyint;
  d.qplus = (T *)c->qplus;
  d.divv = (T *)c->divv;
  d.taurr = (T *)c->taurr;
  d.taurp = (T *)c->taurp;
  d.taupp = (T *)c->taupp;
  d.densr = (T *)c->densr;
  d.energyr = (T *)c->energyr;
  d.radmomp = (T *)c->radmomp;
  d.radmomm = (T *)c->radmomm;
  d.thetamomp = (T *)c->thetamomp;
  d.thetamomm = (T *)c->thetamomm;
  d.sg_accr = (T *)c->sg_accr;
  d.sg_acct = (T *)c->sg_acct;
  d.az_scratch = (T *)c->az_scratch;
  d.rdsum = (T *)c->rdsum;
  d.rt = (const T *)c->rt;
  d.rt64 = c->rt64;
  d.nu = (T *)c->nu;
  d.csmean = c->csmean;
  d.cosF = c->cosF;
  d.sinF = c->sinF;
  d.cosP = (const T *)c->cosP;
  d.cosFt = (const T *)c->cosFt;
  d.sinFt = (const T *)c->sinFt;
  d.sinP = (const T *)c->sinP;
  d.ring_force = c->ring_force;
  d.lostbydisk = c->lostbydisk;
  d.ctl = c->d_ctl;
  a.invdphi = 1.0 / (2.0 * M_PI / (double)c->P.nsec);
  a.dtheta = 2.0 * FARGO_PI / (double)c->P.nsec;
  a.inv_nsec = 1.0 / (double)c->P.nsec;
  a.shear_k = 2.0 * FARGO_PI * FARGO_CFLSECURITY / (double)c->P.nsec;
  a.nr_k1 = pow(c->h.Rinf[1], -1.5) - 1.0;
  a.nr_k2 = c->P.nrad >= 2 ? pow(c->h.Rinf[c->P.nrad - 2], -1.5) - 1.0 : 0.0;
  {
    const double g = c->P.adiabaticindex;
    a.k64[KC_GM1] = g - 1.0;
    a.k64[KC_GGM1] = g * (g - 1.0);
    a.k64[KC_INVDPHI] = a.invdphi;
    a.k64[KC_SGSELF] = 1.0 * c->dp.sgp_rstep * c->dp.sgp_tstep / c->dp.sgp_eps;
    a.k64[KC_DTHETA] = a.dtheta;
    for (int k = 0; k < KC_COUNT; k++) a.k32[k] = (float)a.k64[k];
  }
  if (c->P.nrad >= 3) {
    a.lr01 = log(c->h.Rmed[0] / c->h.Rmed[1]);
    a.lr12 = log(c->h.Rmed[1] / c->h.Rmed[2]);
  }
  a.mode = c->P.sloppy_cfl ? 2 : 0;
  a.az_smem = 0;
  a.az_regs = c->az_regs;
  a.pdl = c->use_pdl ? 1 : 0;
  a.sg_generic = c->sg_generic ? 1 : 0;
  a.rad_maps = c->use_tma ? &c->rad_maps : nullptr;
  a.rad_grid = c->rad_grid;
  {
    static const int bx[4] = {64, 32, 128, 256}, by[4] = {4, 8, 2, 1};
    a.cell_bx = bx[c->cell_block];
    a.cell_by = by[c->cell_block];
  }
  a.az_chunks = c->az_chunks;
  a.rad_col = c->rad_col ? 1 : 0;
  a.cond_handle = 0;
  a.use_cond = 0;
  a.sg.spec_r = c->spec_r;
  a.sg.spec_t = c->spec_t;
  a.sg.spec2_r = c->spec2_r;
  a.sg.spec2_t = c->spec2_t;
  a.sg.khat_r = c->khat_r;
  a.sg.khat_t = c->khat_t;
  a.sg.tw1 = c->tw1;
  a.sg.tw0 = c->tw0;
  a.sg.khat64_r = c->khat64_r;
  a.sg.khat64_t = c->khat64_t;
  a.sg.tw1_64 = c->tw1_64;
  a.sg.tw0_64 = c->tw0_64;
  a.sg.kr = c->kr;
  a.sg.kt = c->kt;
  for (int k = 0; k < 16; k++) {
    a.sg.rad1[k] = c->rad1[k];
    a.sg.rad0[k] = c->rad0[k];
  }
  a.sg.nst1 = c->nst1;
  a.sg.nst0 = c->nst0;
  a.sg.M = c->P.nsec / 2 + 1;
  return a;
}

int dev_alloc(fargo_ctx *c, void **p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return set_err(c, FARGO_ERR_CUDA, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  c->allocs.push_back(*p);
  e = cudaMemsetAsync(*p, 0, bytes, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return set_err(c, FARGO_ERR_CUDA, std::string("cudaMemset: ") + cudaGetErrorString(e));
  return FARGO_OK;
}

// host FP64 -> device T (FP32 fields are converted on the device from an FP64
// staging buffer, so the host side always moves FP64 arrays)
// Enqueues one host -> device transfer on the context's stream; FP32 fields go
// through staging slot `slot` (one field each, so that the transfers of one call
// need no synchronisation between them).  The caller synchronises the stream
// before the host array may change.
static int upload_async(fargo_ctx *c, void *dst, const double *src, size_t n, int slot) {
  if (c->esize == 8) {
    CK(cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyHostToDevice, c->stream));
  } else if (!c->staging || n > c->h.size_grid || slot >= FARGO_STAGING_SLOTS) {
    std::vector<float> tmp(n);
    for (size_t k = 0; k < n; k++) tmp[k] = (float)src[k];
    CK(cudaMemcpyAsync(dst, tmp.data(), n * 4, cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  } else {
    double *st = c->staging + (size_t)slot * c->h.size_grid;
    CK(cudaMemcpyAsync(st, src, n * 8, cudaMemcpyHostToDevice, c->stream));
    launch_convert_from_f64(st, dst, n, (int)c->esize, c->stream);
    CK(cudaGetLastError());
  }
  return FARGO_OK;
}

static int download_async(fargo_ctx *c, double *dst, const void *src, size_t n, int slot) {
  if (c->esize == 8) {
    CK(cudaMemcpyAsync(dst, src, n * 8, cudaMemcpyDeviceToHost, c->stream));
  } else {
    if (slot >= FARGO_STAGING_SLOTS) {  // reuse slot 0 after the transfers before it
      CK(cudaStreamSynchronize(c->stream));
      slot = 0;
    }
    double *st = c->staging + (size_t)slot * c->h.size_grid;
    launch_convert_to_f64(src, st, n, (int)c->esize, c->stream);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(dst, st, n * 8, cudaMemcpyDeviceToHost, c->stream));
  }
  return FARGO_OK;
}

int upload(fargo_ctx *c, void *dst, const double *src, size_t n) {
  int rc = upload_async(c, dst, src, n, 0);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return FARGO_OK;
}

int download(fargo_ctx *c, double *dst, const void *src, size_t n) {
  int rc = download_async(c, dst, src, n, 0);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return FARGO_OK;
}

int read_ctl(fargo_ctx *c) {
  CK(cudaMemcpyAsync(c->pin_ctl, c->d_ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return FARGO_OK;
}

int write_ctl(fargo_ctx *c) {
  fargo_ctl_mirror(*c->pin_ctl);
  CK(cudaMemcpyAsync(c->d_ctl, c->pin_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return FARGO_OK;
}

int check_launch(fargo_ctx *c, const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(c, FARGO_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return FARGO_OK;
}

int device_error(fargo_ctx *c) {
  int e = c->pin_ctl->err;
  if (!e) return FARGO_OK;
  std::string m = "device error:";
  if (e & FARGO_DEVERR_CFL) m += " non-finite or non-positive CFL time step;";
  if (e & FARGO_DEVERR_CAP) m += " substep cap per DT exceeded;";
  if (e & FARGO_DEVERR_NAN) m += " non-finite density;";
  return set_err(c, FARGO_ERR_NUMERIC, m);
}

template <class T>
int build_graph(fargo_ctx *c) {
  KArgs<T> a = make_args<T>(c);
  cudaGraph_t g = nullptr, gp = nullptr;
  CK(cudaGraphCreate(&g, 0));
  LaunchProbe probe;
  std::memset(&probe, 0, sizeof(probe));
  g_probe = &probe;
  // with self-gravity the loop runs rotated: the prefix also runs the first
  // substep's CFL/force kernel and transforms, each substep the next one's
  const bool rot = c->use_rotation && rotation_allowed<T>(a, &c->side);
  const bool ahead = !rot && c->use_sg_ahead && sg_ahead_allowed<T>(a, &c->side);
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  launch_dt_prefix<T>(a, c->stream);
  if (rot) launch_dt_head<T>(a, c->stream, &c->side);
  if (ahead) launch_sg_rows_fwd<T>(a, c->stream);
  g_probe = nullptr;
  CK(cudaStreamEndCapture(c->stream, &gp));
  c->launches_per_dt = probe.count;
  cudaGraphNode_t np, nc;
  CK(cudaGraphAddChildGraphNode(&np, g, nullptr, 0, gp));
  CK(cudaGraphDestroy(gp));
  cudaGraphConditionalHandle h;
  CK(cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  CK(cudaGraphAddNode(&nc, g, &np, nullptr, 1, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  a.cond_handle = (unsigned long long)h;
  a.use_cond = 1;
  // Two substeps per loop iteration when every kernel of a substep is an
  // identity at dt = 0 (no boundary kernel): the loop's turnaround is paid once
  // per two substeps.  A second substep that starts with the DT already done
  // runs with dt = 0 (k_cfl_forces) and changes nothing; k_end counts it apart.
  const bool bc = c->P.open_inner || c->P.non_reflecting || c->P.evanescent;
  const int per_body = (c->use_pad && !rot && !bc) ? 2 : 1;
  CK(cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  probe.count = 0;
  g_probe = &probe;
  for (int k = 0; k < per_body; k++)
    launch_substep_kernels<T>(a, c->stream, SUBK_ALL, c->az_smem, &c->side,
                              rot ? ROT_HEAD_DONE | ROT_NEXT_HEAD : ahead ? SG_AHEAD : 0u);
  g_probe = nullptr;
  CK(cudaStreamEndCapture(c->stream, &body));
  c->launches_per_substep = probe.count / per_body;
  CK(cudaGraphInstantiate(&c->exec, g, cudaGraphInstantiateFlagUseNodePriority));
  c->graph = g;
  c->cond_handle = a.cond_handle;
  return FARGO_OK;
}

// one DT with a host loop (fallback when conditional graph nodes are unavailable)
template <class T>
int run_dt_hostloop(fargo_ctx *c) {
  KArgs<T> a = make_args<T>(c);
  const bool ahead = c->use_sg_ahead && sg_ahead_allowed<T>(a, &c->side);
  launch_dt_prefix<T>(a, c->stream);
  if (ahead) launch_sg_rows_fwd<T>(a, c->stream);
  for (int n = 0; n < FARGO_MAX_SUBSTEPS_PER_DT + 1; n++) {
    launch_substep_kernels<T>(a, c->stream, SUBK_ALL, c->az_smem, &c->side, ahead ? SG_AHEAD : 0u);
    int rc = check_launch(c, "substep");
    if (rc) return rc;
    if ((rc = read_ctl(c))) return rc;
    if (c->pin_ctl->done) break;
  }
  return FARGO_OK;
}

template <class T>
int enqueue_dt(fargo_ctx *c) {
  if (c->use_graph) {
    cudaError_t e = cudaGraphLaunch(c->exec, c->stream);
    if (e != cudaSuccess) return set_err(c, FARGO_ERR_CUDA, std::string("cudaGraphLaunch: ") + cudaGetErrorString(e));
    return FARGO_OK;
  }
  return run_dt_hostloop<T>(c);
}

template <class T>
int init_typed(fargo_ctx *c, const fargo_planet *planets) {
  const fargo_params &p = c->P;
  HostState &h = c->h;
  const size_t sg = h.size_grid, n1 = (size_t)p.nrad + 1;
  const size_t E = sizeof(T);
  Ctl &ctl = *c->pin_ctl;
  std::memset(&ctl, 0, sizeof(Ctl));
  host_init_planets(p, h, planets, c->nb, ctl);
  ctl.DT = p.dt;
  // device arrays
  void **fields[] = {&c->dens, &c->vrad, &c->vtheta, &c->energy, &c->pressure, &c->temperature, &c->potential,
                     &c->vradint, &c->vthetaint, &c->energyint, &c->qplus, &c->divv, &c->taurr, &c->taurp,
                     &c->taupp, &c->densr, &c->energyr, &c->radmomp, &c->radmomm, &c->thetamomp, &c->thetamomm};
  int rc;
  for (void **f : fields)
    if ((rc = dev_alloc(c, f, sg * E))) return rc;
  if (p.adiabatic && (rc = dev_alloc(c, &c->cs, sg * E))) return rc;
  // FP64: the reciprocals of the neighbour density sums, shared by the substep's
  // source, viscous-update and artificial-viscosity divides
  if (E == 8 && (rc = dev_alloc(c, &c->rdsum, 2 * sg * E))) return rc;
  if ((rc = dev_alloc(c, &c->rt, (size_t)RT_COUNT * n1 * E))) return rc;
  if ((rc = dev_alloc(c, (void **)&c->rt64, (size_t)RT_COUNT * n1 * 8))) return rc;
  if ((rc = dev_alloc(c, &c->nu, 2 * n1 * E))) return rc;  // nu, then 0.5 / nu (Qplus)
  if ((rc = dev_alloc(c, (void **)&c->csmean, n1 * 8))) return rc;
  if ((rc = dev_alloc(c, (void **)&c->cosF, (size_t)p.nsec * 8))) return rc;
  if ((rc = dev_alloc(c, (void **)&c->sinF, (size_t)p.nsec * 8))) return rc;
  if ((rc = dev_alloc(c, &c->cosP, (size_t)p.nsec * E))) return rc;
  if ((rc = dev_alloc(c, &c->sinP, (size_t)p.nsec * E))) return rc;
  if ((rc = dev_alloc(c, &c->cosFt, (size_t)p.nsec * E))) return rc;
  if ((rc = dev_alloc(c, &c->sinFt, (size_t)p.nsec * E))) return rc;
  if ((rc = dev_alloc(c, (void **)&c->ring_force, n1 * (FARGO_MAXPL + 1) * 2 * 8))) return rc;
  if ((rc = dev_alloc(c, (void **)&c->lostbydisk, (size_t)p.nsec * 8))) return rc;
  if (c->esize == 4 && (rc = dev_alloc(c, (void **)&c->staging, FARGO_STAGING_SLOTS * sg * 8))) return rc;
  // azimuthal transport ring buffers: shared memory when they fit
  {
    int dev = 0, maxsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&maxsm, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    size_t need = (size_t)AZ_NARR_HOST * p.nsec * E, need4 = (size_t)13 * p.nsec * E;
    const char *fg = std::getenv("FARGO_AZ_GLOBAL");  // force the global-memory ring buffers
    const bool force_global = fg && fg[0] == '1';
    const bool force_generic = force_global || c->az_generic;  // the barrier-per-phase kernel
    // register-blocked kernel when its ring fits in shared memory (chunks of four
    // cells over at most 768 FP32 / 512 FP64 threads)
    if (!force_generic && p.nsec % 4 == 0 && need4 + 1024 <= (size_t)maxsm) {
      c->az_smem = need4;
      c->az_regs = 1;
      CK(prepare_kernels<T>(need4, 1));
    } else if (!force_global && need + 1024 <= (size_t)maxsm) {
      c->az_smem = need;
      CK(prepare_kernels<T>(need, 0));
    } else {
      c->az_smem = 0;
      CK(prepare_kernels<T>(0, 0));
      if ((rc = dev_alloc(c, &c->az_scratch, (size_t)p.nrad * AZ_NARR_HOST * p.nsec * E))) return rc;
    }
  }
  // TMA maps of the radial transport's input fields
  if (c->want_tma) make_rad_maps<T>(c);
  CK(cudaStreamSynchronize(c->stream));
  // density first: self-gravity set-up needs it
  if ((rc = upload(c, c->dens, h.Dens.data(), sg))) return rc;
  std::vector<double> tmpd;
  if (p.self_gravity) {
    const int n0 = 2 * p.nrad, M = p.nsec / 2 + 1;
    c->nst1 = sg_radices(p.nsec, c->rad1);
    c->nst0 = sg_radices(n0, c->rad0);
    if (c->nst1 < 0 || c->nst0 < 0)
      return set_err(c, FARGO_ERR_INVALID, "self-gravity needs NSEC and 2*NRAD of the form 2^a 3^b");
    host_sg_kernel(p, h, c->dp);
    // per-step spectra and twiddles in the field type; the FP64 set-up buffers
    // are the same ones in the FP64 mode
    const size_t cx = 2 * E;
    if ((rc = dev_alloc(c, &c->spec_r, (size_t)M * p.nrad * cx))) return rc;
    if ((rc = dev_alloc(c, &c->spec_t, (size_t)M * p.nrad * cx))) return rc;
    if ((rc = dev_alloc(c, &c->spec2_r, (size_t)M * p.nrad * cx))) return rc;
    if ((rc = dev_alloc(c, &c->spec2_t, (size_t)M * p.nrad * cx))) return rc;
    if ((rc = dev_alloc(c, &c->khat_r, (size_t)M * n0 * cx))) return rc;
    if ((rc = dev_alloc(c, &c->khat_t, (size_t)M * n0 * cx))) return rc;
    if ((rc = dev_alloc(c, &c->tw1, (size_t)p.nsec * cx))) return rc;
    if ((rc = dev_alloc(c, &c->tw0, (size_t)n0 * cx))) return rc;
    if (E == 8) {
      c->khat64_r = (double2 *)c->khat_r;
      c->khat64_t = (double2 *)c->khat_t;
      c->tw1_64 = (double2 *)c->tw1;
      c->tw0_64 = (double2 *)c->tw0;
    } else {
      if ((rc = dev_alloc(c, (void **)&c->khat64_r, (size_t)M * n0 * 16))) return rc;
      if ((rc = dev_alloc(c, (void **)&c->khat64_t, (size_t)M * n0 * 16))) return rc;
      if ((rc = dev_alloc(c, (void **)&c->tw1_64, (size_t)p.nsec * 16))) return rc;
      if ((rc = dev_alloc(c, (void **)&c->tw0_64, (size_t)n0 * 16))) return rc;
    }
    if ((rc = dev_alloc(c, (void **)&c->kr, (size_t)n0 * p.nsec * 8))) return rc;
    if ((rc = dev_alloc(c, (void **)&c->kt, (size_t)n0 * p.nsec * 8))) return rc;
    if ((rc = dev_alloc(c, &c->sg_accr, sg * E))) return rc;
    if ((rc = dev_alloc(c, &c->sg_acct, sg * E))) return rc;
    auto twiddles = [](int n) {
      std::vector<double> t(2 * (size_t)n);
      for (int k = 0; k < n; k++) {
        long double ang = 2.0L * 3.141592653589793238462643383279502884L * (long double)k / (long double)n;
        t[2 * k] = (double)cosl(ang);
        t[2 * k + 1] = (double)(-sinl(ang));
      }
      return t;
    };
    std::vector<double> t1 = twiddles(p.nsec), t0 = twiddles(n0);
    CK(cudaMemcpy(c->tw1_64, t1.data(), t1.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->tw0_64, t0.data(), t0.size() * 8, cudaMemcpyHostToDevice));
    if (E == 4) {
      std::vector<float> f1(t1.begin(), t1.end()), f0(t0.begin(), t0.end());
      CK(cudaMemcpy(c->tw1, f1.data(), f1.size() * 4, cudaMemcpyHostToDevice));
      CK(cudaMemcpy(c->tw0, f0.data(), f0.size() * 4, cudaMemcpyHostToDevice));
    }
    CK(cudaMemcpy(c->kr, h.Kr.data(), h.Kr.size() * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->kt, h.Kt.data(), h.Kt.size() * 8, cudaMemcpyHostToDevice));
    CK(prepare_sg_kernels<T>(p.nsec, n0));
    // ring table rows the SG kernels read
    std::vector<double> tab;
    host_ring_table(p, h, c->dp, tab);  // uses only mesh rows at this point
    CK(cudaMemcpy(c->rt64, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice));
    if ((rc = upload(c, c->rt, tab.data(), tab.size()))) return rc;
    KArgs<T> a = make_args<T>(c);
    a.P = c->dp;
    launch_sg_kernel_spectra<T>(a, c->stream);
    if ((rc = check_launch(c, "sg kernel spectra"))) return rc;
    launch_selfgravity<T>(a, c->stream);
    if ((rc = check_launch(c, "sg set-up"))) return rc;
    std::vector<double> accr(sg);
    if ((rc = download(c, accr.data(), c->sg_accr, sg))) return rc;
    std::vector<double> axi(p.nrad + 1, 0.0);
    for (int i = 0; i < p.nrad; i++) {
      double s = 0.0;
      for (int j = 0; j < p.nsec; j++) s += accr[(size_t)i * p.nsec + j];
      axi[i] = s / (double)p.nsec;
    }
    host_init_planets_sg(p, h, axi, ctl);
  }
  host_init_euler(p, h, c->dp, ctl);
  std::vector<double> tab;
  host_ring_table(p, h, c->dp, tab);
  CK(cudaMemcpy(c->rt64, tab.data(), tab.size() * 8, cudaMemcpyHostToDevice));
  if ((rc = upload(c, c->rt, tab.data(), tab.size()))) return rc;
  if ((rc = upload(c, c->nu, h.nu.data(), n1))) return rc;
  {
    // 0.5 / nu of the heating term, as the kernels divide it in the field type (in
    // double from the float value for FP32: the same correctly rounded quotient)
    std::vector<double> hnu(n1);
    for (size_t k = 0; k < n1; k++) {
      const double v = E == 4 ? (double)(float)h.nu[k] : h.nu[k];
      hnu[k] = v != 0.0 ? 0.5 / v : 0.0;
    }
    if ((rc = upload(c, (char *)c->nu + n1 * E, hnu.data(), n1))) return rc;
  }
  CK(cudaMemcpy(c->csmean, h.cs_mean.data(), n1 * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->cosF, h.cosF.data(), (size_t)p.nsec * 8, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(c->sinF, h.sinF.data(), (size_t)p.nsec * 8, cudaMemcpyHostToDevice));
  if ((rc = upload(c, c->cosP, h.cosP.data(), p.nsec))) return rc;
  if ((rc = upload(c, c->sinP, h.sinP.data(), p.nsec))) return rc;
  if ((rc = upload(c, c->cosFt, h.cosF.data(), p.nsec))) return rc;
  if ((rc = upload(c, c->sinFt, h.sinF.data(), p.nsec))) return rc;
  if ((rc = upload(c, c->vrad, h.Vrad.data(), sg))) return rc;
  if ((rc = upload(c, c->vtheta, h.Vtheta.data(), sg))) return rc;
  if ((rc = upload(c, c->energy, h.Energy.data(), sg))) return rc;
  if ((rc = upload(c, c->pressure, h.Pressure.data(), sg))) return rc;
  if ((rc = upload(c, c->temperature, h.Temperature.data(), sg))) return rc;
  if (p.adiabatic && (rc = upload(c, c->cs, h.SoundSpeed.data(), sg))) return rc;
  ctl.PhysicalTime = 0.0;
  ctl.PhysicalTimeInitial = 0.0;
  ctl.OmegaFrame = h.OmegaFrame;
  fargo_planet_params(ctl, c->dp, ctl.PhysicalTime);
  if ((rc = write_ctl(c))) return rc;
  // the SG spectra are no longer needed on the host
  h.Kr.clear();
  h.Kt.clear();
  if (c->use_graph) {
    rc = build_graph<T>(c);
    if (rc != FARGO_OK) {
      // conditional graph nodes unavailable: fall back to the host loop
      cudaGetLastError();
      c->use_graph = false;
      c->err = "graph fallback: " + c->err;
    }
  }
  return FARGO_OK;
}

template <class T>
int substep_typed(fargo_ctx *c, int which, double dt) {
  KArgs<T> a = make_args<T>(c);
  int rc;
  if ((rc = read_ctl(c))) return rc;
  c->pin_ctl->dt = dt;
  c->pin_ctl->dt_sub = dt;
  c->pin_ctl->sloppy_dt = dt;
  if ((rc = write_ctl(c))) return rc;
  unsigned mask = 0;
  switch (which) {
    case FARGO_SUB_BOUNDARY: launch_boundaries<T>(a, c->stream); break;
    case FARGO_SUB_SOURCE: mask = SUBK_SG | SUBK_SOURCE; break;
    case FARGO_SUB_ENERGY:
      if (!c->P.adiabatic) return set_err(c, FARGO_ERR_INVALID, "no energy equation");
      mask = SUBK_ENERGY;
      break;
    case FARGO_SUB_TRANSPORT: mask = SUBK_TRANSPORT; break;
    case FARGO_SUB_TEMPERATURE: mask = SUBK_TEMPERATURE; break;
    case FARGO_SUB_SOUNDSPEED:
      if (c->P.adiabatic) {
        KArgs<T> b = a;
        launch_dt_prefix<T>(b, c->stream);  // resets the DT counters and computes cs
      }
      break;
    case FARGO_SUB_POTENTIAL:
      a.mode = 3;
      mask = SUBK_CFL_FORCES;
      break;
    default: return set_err(c, FARGO_ERR_INVALID, "unknown substep");
  }
  if (!c->P.self_gravity) mask &= ~SUBK_SG;
  if (mask) launch_substep_kernels<T>(a, c->stream, mask, c->az_smem);
  if ((rc = check_launch(c, "substep"))) return rc;
  CK(cudaStreamSynchronize(c->stream));
  return FARGO_OK;
}

template <class T>
int substep_full_typed(fargo_ctx *c, double dt) {
  KArgs<T> a = make_args<T>(c);
  int rc;
  if ((rc = read_ctl(c))) return rc;
  Ctl &k = *c->pin_ctl;
  k.sloppy_dt = dt;
  k.DT = dt;
  k.dtemp = 0.0;
  k.nsub_dt = 0;
  k.done = 0;
  if ((rc = write_ctl(c))) return rc;
  a.mode = 2;
  launch_substep_kernels<T>(a, c->stream, SUBK_ALL, c->az_smem);
  if ((rc = check_launch(c, "substep_full"))) return rc;
  if ((rc = read_ctl(c))) return rc;
  c->pin_ctl->DT = c->P.dt;
  if ((rc = write_ctl(c))) return rc;
  return device_error(c);
}

template <class T>
int cfl_typed(fargo_ctx *c, double deltaT, int *cfl) {
  int rc;
  if ((rc = read_ctl(c))) return rc;
  const double saved = c->pin_ctl->DT;
  c->pin_ctl->DT = deltaT;
  if ((rc = write_ctl(c))) return rc;
  launch_cfl_only<T>(make_args<T>(c), c->stream);
  if ((rc = check_launch(c, "cfl"))) return rc;
  if ((rc = read_ctl(c))) return rc;
  *cfl = c->pin_ctl->cfl;
  c->pin_ctl->DT = saved;
  c->pin_ctl->err = 0;
  c->pin_ctl->done = 0;
  return write_ctl(c);
}

// Per-kernel device time of reps substeps, launched one by one with events.
template <class T>
int time_kernels_typed(fargo_ctx *c, int reps, std::vector<double> &ms) {
  KArgs<T> a = make_args<T>(c);
  LaunchProbe probe;
  std::memset(&probe, 0, sizeof(probe));
  probe.nev = 96;
  for (int k = 0; k < probe.nev; k++) CK(cudaEventCreate(&probe.ev[k]));
  cudaEvent_t start;
  CK(cudaEventCreate(&start));
  int rc = FARGO_OK;
  for (int r = 0; r < reps && rc == FARGO_OK; r++) {
    launch_dt_prefix<T>(a, c->stream);  // a fresh DT per repetition keeps dtemp < DT
    CK(cudaEventRecord(start, c->stream));
    probe.n = 0;
    probe.count = 0;
    g_probe = &probe;
    launch_substep_kernels<T>(a, c->stream, SUBK_ALL, c->az_smem);
    g_probe = nullptr;
    rc = check_launch(c, "timed substep");
    if (rc) break;
    CK(cudaStreamSynchronize(c->stream));
    if (ms.empty()) {
      ms.assign(probe.n, 0.0);
      c->kernel_names.assign(probe.name, probe.name + probe.n);
    }
    cudaEvent_t prev = start;
    for (int k = 0; k < probe.n && k < (int)ms.size(); k++) {
      float t = 0.f;
      CK(cudaEventElapsedTime(&t, prev, probe.ev[k]));
      ms[k] += t / reps;
      prev = probe.ev[k];
    }
  }
  for (int k = 0; k < probe.nev; k++) cudaEventDestroy(probe.ev[k]);
  cudaEventDestroy(start);
  if (rc) return rc;
  // the timed substeps moved the clock; keep the DT bookkeeping consistent
  if ((rc = read_ctl(c))) return rc;
  return device_error(c);
}

void *field_ptr(fargo_ctx *c, int which) {
  switch (which) {
    case FARGO_FIELD_DENS: return c->dens;
    case FARGO_FIELD_VRAD: return c->vrad;
    case FARGO_FIELD_VTHETA: return c->vtheta;
    case FARGO_FIELD_ENERGY: return c->energy;
    case FARGO_FIELD_TEMPERATURE: return c->temperature;
    case FARGO_FIELD_PRESSURE: return c->pressure;
    case FARGO_FIELD_SOUNDSPEED: return c->cs;
    case FARGO_FIELD_POTENTIAL: return c->potential;
    case FARGO_FIELD_QPLUS: return c->qplus;
    case FARGO_FIELD_DIVERGENCE: return c->divv;
    case FARGO_FIELD_SG_ACCR: return c->sg_accr;
    case FARGO_FIELD_SG_ACCT: return c->sg_acct;
  }
  return nullptr;
}

}  // namespace

#define DISPATCH(c, fn, ...) ((c)->precision == FARGO_FP64 ? fn<double>(__VA_ARGS__) : fn<float>(__VA_ARGS__))

extern "C" {

static bool env_on(const char *name) {
  const char *v = std::getenv(name);
  return v && v[0] == '1';
}

void fargo_variant_default(fargo_variant *v) {
  if (!v) return;
  v->graph = env_on("FARGO_NO_GRAPH") ? 0 : 1;
  v->pdl = env_on("FARGO_NO_PDL") ? 0 : 1;
  v->pad = env_on("FARGO_NO_PAD") ? 0 : 1;
  v->sg_ahead = env_on("FARGO_NO_SG_AHEAD") ? 0 : 1;
  v->rotate = env_on("FARGO_ROTATE") ? 1 : 0;
  v->az_generic = env_on("FARGO_AZ_GENERIC") ? 1 : 0;
  const char *pr = std::getenv("FARGO_PRIO");
  v->priority = pr ? std::atoi(pr) : 0;
  const char *cb = std::getenv("FARGO_CELL_BLOCK");
  v->cell_block = cb ? std::atoi(cb) : 0;
  v->rad_tma = env_on("FARGO_NO_TMA") ? 0 : 1;
  v->az_chunks = env_on("FARGO_AZ_CHUNKS2") ? 2 : 1;
  const char *rc = std::getenv("FARGO_RAD_COL");
  v->rad_col = rc ? (std::atoi(rc) ? 1 : 0) : -1;
}

int fargo_ctx_create(const fargo_params *p, const fargo_planet *planets, int nb, int precision, void *stream,
                     fargo_ctx **out) {
  return fargo_ctx_create_variant(p, planets, nb, precision, stream, nullptr, out);
}

int fargo_ctx_create_variant(const fargo_params *p, const fargo_planet *planets, int nb, int precision, void *stream,
                             const fargo_variant *variant, fargo_ctx **out) {
  if (!p || !out || nb < 0 || nb > FARGO_MAXPL || (nb > 0 && !planets)) return FARGO_ERR_INVALID;
  fargo_variant v;
  if (variant) v = *variant;
  else fargo_variant_default(&v);
  if (v.priority < 0 || v.priority > 2) return FARGO_ERR_INVALID;
  if (v.cell_block < 0 || v.cell_block > 3 || v.az_chunks < 1 || v.az_chunks > 2) return FARGO_ERR_INVALID;
  if (v.rad_col < -1 || v.rad_col > 1) return FARGO_ERR_INVALID;
  if (precision != FARGO_FP64 && precision != FARGO_FP32_BULK) return FARGO_ERR_INVALID;
  if (p->nrad < 8 || p->nsec < 8 || !p->is_disk || !(p->dt > 0.0)) return FARGO_ERR_INVALID;
  fargo_ctx *c = new fargo_ctx();
  c->P = *p;
  c->nb = nb;
  c->precision = precision;
  c->esize = precision == FARGO_FP64 ? 8 : 4;
  c->dp = host_dev_params(*p, nb);
  c->use_graph = v.graph != 0;
  c->use_pdl = v.pdl != 0;
  c->use_rotation = v.rotate != 0;
  c->use_sg_ahead = v.sg_ahead != 0;
  c->use_pad = v.pad != 0;
  c->az_generic = v.az_generic != 0;
  c->want_tma = v.rad_tma != 0;
  c->cell_block = v.cell_block;
  c->az_chunks = v.az_chunks;
  // the column march by default where it measured faster: FP32-bulk grids with at
  // least 65536 column chunks (3072 sectors x 1024 rings: 64 against 85 us); a
  // 768 x 256 grid gives it 48 CTAs, and FP64 is bound by its pipe either way
  c->rad_col = v.rad_col < 0 ? (precision == FARGO_FP32_BULK &&
                                (long)p->nsec * ((p->nrad + RADC_RINGS - 1) / RADC_RINGS) >= 65536)
                             : v.rad_col != 0;
  c->sg_generic = env_on("FARGO_SG_GENERIC");  // a parity-test switch, not a variant
  // stream priorities: 0 all equal; 1 the hydro chain and the planets above the
  // self-gravity transforms; 2 the transforms above the rest.  The caller's
  // stream keeps its own priority.
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  const int p_main = v.priority == 1 ? prio_hi : prio_lo, p_sg = v.priority == 2 ? prio_hi : prio_lo;
  int rc = FARGO_OK;
  cudaError_t e;
  if (stream) {
    c->stream = (cudaStream_t)stream;
  } else {
    e = cudaStreamCreateWithPriority(&c->stream, cudaStreamNonBlocking, p_main);
    if (e != cudaSuccess) {
      delete c;
      return FARGO_ERR_CUDA;
    }
    c->own_stream = true;
  }
  e = cudaStreamCreateWithPriority(&c->side.s, cudaStreamNonBlocking, p_main);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->side.fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->side.join, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->side.s2, cudaStreamNonBlocking, p_sg);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->side.fork2, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->side.join2, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMallocHost((void **)&c->pin_ctl, sizeof(Ctl));
  if (e == cudaSuccess) e = cudaMalloc((void **)&c->d_ctl, sizeof(Ctl));
  if (e != cudaSuccess) {
    fargo_ctx_destroy(c);
    return FARGO_ERR_CUDA;
  }
  host_fill_mesh(*p, c->h);
  host_init_density_energy(*p, c->h);
  rc = DISPATCH(c, init_typed, c, planets);
  if (rc != FARGO_OK) {
    std::fprintf(stderr, "fargo_ctx_create: %s\n", c->err.c_str());
    fargo_ctx_destroy(c);
    return rc;
  }
  *out = c;
  return FARGO_OK;
}

void fargo_ctx_destroy(fargo_ctx *c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->exec) cudaGraphExecDestroy(c->exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  for (void *p : c->allocs) cudaFree(p);
  if (c->d_ctl) cudaFree(c->d_ctl);
  if (c->pin_ctl) cudaFreeHost(c->pin_ctl);
  if (c->side.s) cudaStreamSynchronize(c->side.s);
  if (c->side.fork) cudaEventDestroy(c->side.fork);
  if (c->side.join) cudaEventDestroy(c->side.join);
  if (c->side.s) cudaStreamDestroy(c->side.s);
  if (c->side.s2) cudaStreamSynchronize(c->side.s2);
  if (c->side.fork2) cudaEventDestroy(c->side.fork2);
  if (c->side.join2) cudaEventDestroy(c->side.join2);
  if (c->side.s2) cudaStreamDestroy(c->side.s2);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

const char *fargo_last_error(const fargo_ctx *c) { return c ? c->err.c_str() : "no context"; }

// All requested fields enqueued back to back (FP32 fields: one conversion
// launch through the staging slots), one synchronisation per call
int fargo_get_fields(fargo_ctx *c, double *dens, double *vrad, double *vtheta, double *energy, double *temperature) {
  if (!c) return FARGO_ERR_STATE;
  const size_t n = c->h.size_grid;
  double *dst[5] = {dens, vrad, vtheta, energy, temperature};
  const void *src[5] = {c->dens, c->vrad, c->vtheta, c->energy, c->temperature};
  if (c->esize == 4 && c->staging) {
    ConvFields p{};
    double *host[5];
    for (int k = 0; k < 5; k++)
      if (dst[k]) {
        p.src[p.nf] = src[k];
        p.dst[p.nf] = c->staging + (size_t)p.nf * n;
        host[p.nf++] = dst[k];
      }
    if (p.nf) launch_convert_to_f64_multi(p, n, 4, c->stream);
    CK(cudaGetLastError());
    for (int f = 0; f < p.nf; f++)
      CK(cudaMemcpyAsync(host[f], p.dst[f], n * 8, cudaMemcpyDeviceToHost, c->stream));
  } else {
    int rc, slot = 0;
    for (int k = 0; k < 5; k++)
      if (dst[k] && (rc = download_async(c, dst[k], src[k], n, slot++))) return rc;
  }
  CK(cudaStreamSynchronize(c->stream));
  return FARGO_OK;
}

int fargo_set_fields(fargo_ctx *c, const double *dens, const double *vrad, const double *vtheta, const double *energy) {
  if (!c) return FARGO_ERR_STATE;
  const size_t n = c->h.size_grid;
  const double *src[4] = {dens, vrad, vtheta, energy};
  void *dst[4] = {c->dens, c->vrad, c->vtheta, c->energy};
  if (c->esize == 4 && c->staging) {
    ConvFields p{};
    for (int k = 0; k < 4; k++)
      if (src[k]) {
        double *st = c->staging + (size_t)p.nf * n;
        CK(cudaMemcpyAsync(st, src[k], n * 8, cudaMemcpyHostToDevice, c->stream));
        p.src[p.nf] = st;
        p.dst[p.nf++] = dst[k];
      }
    if (p.nf) launch_convert_from_f64_multi(p, n, 4, c->stream);
    CK(cudaGetLastError());
  } else {
    int rc, slot = 0;
    for (int k = 0; k < 4; k++)
      if (src[k] && (rc = upload_async(c, dst[k], src[k], n, slot++))) return rc;
  }
  CK(cudaStreamSynchronize(c->stream));
  return FARGO_OK;
}

int fargo_get_field(fargo_ctx *c, int which, double *host) {
  if (!c || !host) return FARGO_ERR_STATE;
  void *p = field_ptr(c, which);
  if (which == FARGO_FIELD_SOUNDSPEED && !p) {
    // isothermal: the ring sound speed broadcast over the sectors
    const HostState &h = c->h;
    for (size_t q = 0; q < h.size_grid; q++) host[q] = q < h.SoundSpeed.size() ? h.SoundSpeed[q] : 0.0;
    return FARGO_OK;
  }
  if (!p) return set_err(c, FARGO_ERR_INVALID, "field not available in this configuration");
  int rc = download(c, host, p, c->h.size_grid);
  if (rc || which != FARGO_FIELD_POTENTIAL || c->nb == 0) return rc;
  // the device array holds the planet part; the star term (direct + indirect,
  // src/Kernels.cu:1246-1250) is evaluated by its consumer, and here on the host
  if ((rc = read_ctl(c))) return rc;
  const HostState &h = c->h;
  const double ix = c->pin_ctl->ind_x, iy = c->pin_ctl->ind_y;
  for (int i = 0; i < c->P.nrad; i++)
    for (int j = 0; j < c->P.nsec; j++) {
      const double x = h.Rmed[i] * h.cosP[j], y = h.Rmed[i] * h.sinP[j];
      double pot = -h.invRmed[i];
      pot -= ix * x + iy * y;
      host[(size_t)i * c->P.nsec + j] += pot;
    }
  return FARGO_OK;
}

int fargo_get_field_device(fargo_ctx *c, int which, double *dev) {
  if (!c || !dev) return FARGO_ERR_STATE;
  void *p = field_ptr(c, which);
  if (!p || which == FARGO_FIELD_POTENTIAL)
    return set_err(c, FARGO_ERR_INVALID, "field not held on the device in this configuration");
  const size_t n = c->h.size_grid;
  if (c->esize == 8) {
    CK(cudaMemcpyAsync(dev, p, n * 8, cudaMemcpyDeviceToDevice, c->stream));
  } else {
    launch_convert_to_f64(p, dev, n, (int)c->esize, c->stream);
    CK(cudaGetLastError());
  }
  CK(cudaStreamSynchronize(c->stream));
  return FARGO_OK;
}

int fargo_get_planets(fargo_ctx *c, fargo_planet *out, int cap, int *nb) {
  if (!c || !nb) return FARGO_ERR_STATE;
  int rc;
  if ((rc = read_ctl(c))) return rc;
  const Ctl &k = *c->pin_ctl;
  *nb = k.nb;
  for (int i = 0; i < k.nb && i < cap; i++) {
    out[i].x = k.x[i];
    out[i].y = k.y[i];
    out[i].vx = k.vx[i];
    out[i].vy = k.vy[i];
    out[i].mass = k.mass[i];
    out[i].acc = k.acc[i];
    out[i].feel_disk = k.feeldisk[i];
    out[i].feel_others = k.feelothers[i];
  }
  return FARGO_OK;
}

int fargo_get_scalars(fargo_ctx *c, fargo_scalars *s) {
  if (!c || !s) return FARGO_ERR_STATE;
  int rc;
  if ((rc = read_ctl(c))) return rc;
  const Ctl &k = *c->pin_ctl;
  s->physical_time = k.PhysicalTime;
  s->omega_frame = k.OmegaFrame;
  s->lost_mass = k.LostMass;
  s->last_dt = k.dt_sub;
  s->padded_substeps = k.padded;
  s->substeps = k.substeps;
  s->last_cfl = k.cfl;
  s->nb = k.nb;
  s->launches_per_substep = c->launches_per_substep;
  s->launches_per_dt = c->launches_per_dt;
  return FARGO_OK;
}

int fargo_get_mesh(fargo_ctx *c, double *rinf, double *rmed, double *rsup, double *surf) {
  if (!c) return FARGO_ERR_STATE;
  const size_t n = (size_t)c->P.nrad + 1;
  if (rinf) std::memcpy(rinf, c->h.Rinf.data(), n * 8);
  if (rmed) std::memcpy(rmed, c->h.Rmed.data(), n * 8);
  if (rsup) std::memcpy(rsup, c->h.Rsup.data(), n * 8);
  if (surf) std::memcpy(surf, c->h.Surf.data(), n * 8);
  return FARGO_OK;
}

int fargo_step_DT(fargo_ctx *c, int *nsub) {
  if (!c) return FARGO_ERR_STATE;
  int rc = DISPATCH(c, enqueue_dt, c);
  if (rc) return rc;
  if ((rc = read_ctl(c))) return rc;
  if (nsub) *nsub = c->pin_ctl->nsub_dt;
  return device_error(c);
}

int fargo_disk_view(fargo_ctx *c, DiskView *v) {
  if (!c || !v) return FARGO_ERR_STATE;
  int rc = read_ctl(c);
  if (rc) return rc;
  v->dens = c->dens;
  v->vrad = c->vrad;
  v->vtheta = c->vtheta;
  v->esize = (int)c->esize;
  v->nrad = c->P.nrad;
  v->nsec = c->P.nsec;
  v->stream = (void *)c->stream;
  v->rmed = c->h.Rmed.data();
  v->surf = c->h.Surf.data();
  v->planet_phi = c->nb > 0 ? std::atan2(c->pin_ctl->y[0], c->pin_ctl->x[0]) : 0.0;
  if (!c->lx_rmed) {
    const size_t n1 = (size_t)c->P.nrad + 1;
    if ((rc = dev_alloc(c, (void **)&c->lx_rmed, n1 * 8))) return rc;
    if ((rc = dev_alloc(c, (void **)&c->lx_surf, n1 * 8))) return rc;
    if ((rc = dev_alloc(c, (void **)&c->lx_ring, 3 * n1 * 8))) return rc;
    if ((rc = dev_alloc(c, &c->lx_cand, (size_t)c->P.nrad * c->P.nsec * c->esize))) return rc;
    CK(cudaMemcpy(c->lx_rmed, c->h.Rmed.data(), n1 * 8, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(c->lx_surf, c->h.Surf.data(), n1 * 8, cudaMemcpyHostToDevice));
  }
  v->rmed_dev = c->lx_rmed;
  v->surf_dev = c->lx_surf;
  v->ring = c->lx_ring;
  v->cand = c->lx_cand;
  return FARGO_OK;
}

int fargo_run_async(fargo_ctx *c, int ndt) {
  if (!c || ndt < 0) return FARGO_ERR_STATE;
  for (int k = 0; k < ndt; k++) {
    int rc = DISPATCH(c, enqueue_dt, c);
    if (rc) return rc;
  }
  return FARGO_OK;
}

int fargo_sync(fargo_ctx *c) {
  if (!c) return FARGO_ERR_STATE;
  CK(cudaStreamSynchronize(c->stream));
  return FARGO_OK;
}

int fargo_run(fargo_ctx *c, int ndt, long long *nsub) {
  if (!c) return FARGO_ERR_STATE;
  int rc;
  if ((rc = read_ctl(c))) return rc;
  const long long s0 = c->pin_ctl->substeps;
  if ((rc = fargo_run_async(c, ndt))) return rc;
  if ((rc = read_ctl(c))) return rc;
  if (nsub) *nsub = c->pin_ctl->substeps - s0;
  return device_error(c);
}

int fargo_substep_full(fargo_ctx *c, double dt) {
  if (!c || !(dt > 0.0)) return FARGO_ERR_INVALID;
  return DISPATCH(c, substep_full_typed, c, dt);
}

int fargo_substep(fargo_ctx *c, int which, double dt) {
  if (!c) return FARGO_ERR_STATE;
  return DISPATCH(c, substep_typed, c, which, dt);
}

int fargo_condition_cfl(fargo_ctx *c, double deltaT, int *cfl) {
  if (!c || !cfl) return FARGO_ERR_STATE;
  return DISPATCH(c, cfl_typed, c, deltaT, cfl);
}

int fargo_write_outputs(fargo_ctx *c, int index) {
  if (!c) return FARGO_ERR_STATE;
  const fargo_params &p = c->P;
  const size_t n = c->h.size_grid, nout = (size_t)p.nrad * p.nsec;
  std::vector<double> buf(n);
  std::string dir = p.outputdir;
  struct Item {
    int on;
    int field;
    const char *name;
  } items[] = {{p.write_density, FARGO_FIELD_DENS, "dens"},
               {p.write_velocity, FARGO_FIELD_VRAD, "vrad"},
               {p.write_velocity, FARGO_FIELD_VTHETA, "vtheta"},
               {p.write_energy, FARGO_FIELD_ENERGY, "energy"},
               {p.write_temperature, FARGO_FIELD_TEMPERATURE, "temperature"},
               {p.write_divv, FARGO_FIELD_DIVERGENCE, "divergence"},
               {p.write_qplus, FARGO_FIELD_QPLUS, "qplus"}};
  int rc;
  for (const Item &it : items) {
    if (!it.on) continue;
    if ((rc = fargo_get_field(c, it.field, buf.data()))) return rc;
    if ((rc = host_write_field(dir, it.name, index, buf.data(), nout)))
      return set_err(c, rc, std::string("cannot write ") + it.name);
  }
  fargo_planet pl[FARGO_MAXPL];
  int nb = 0;
  if ((rc = fargo_get_planets(c, pl, FARGO_MAXPL, &nb))) return rc;
  fargo_scalars s;
  if ((rc = fargo_get_scalars(c, &s))) return rc;
  for (int k = 0; k < nb; k++)
    if ((rc = host_write_planet_row(dir, k, index, pl[k], s.lost_mass, s.physical_time, s.omega_frame)))
      return set_err(c, rc, "cannot write planet file");
  return FARGO_OK;
}

int fargo_time_substep_kernels(fargo_ctx *c, int reps, double *ms_per_kernel, int cap, int *nkernels) {
  if (!c || reps < 1 || !nkernels) return FARGO_ERR_INVALID;
  std::vector<double> ms;
  int rc = DISPATCH(c, time_kernels_typed, c, reps, ms);
  if (rc) return rc;
  *nkernels = (int)ms.size();
  for (int k = 0; k < (int)ms.size() && k < cap; k++) ms_per_kernel[k] = ms[k];
  return FARGO_OK;
}

const char *fargo_substep_kernel_name(const fargo_ctx *c, int k) {
  if (!c || k < 0 || k >= (int)c->kernel_names.size()) return nullptr;
  return c->kernel_names[k].c_str();
}

int fargo_write_dims(fargo_ctx *c) {
  if (!c) return FARGO_ERR_STATE;
  int rc;
  if ((rc = host_write_used_rad(c->P, c->h))) return set_err(c, rc, "cannot write used_rad.dat");
  if ((rc = host_write_dims(c->P, c->nb))) return set_err(c, rc, "cannot write dims.dat");
  return FARGO_OK;
}

// UpdateLog src/Force.cu:19-84: smoothing and Hill radius of each planet as
// there (RocheSmoothing or Compute_smoothing), ComputeForce, the rows.
int fargo_update_log(fargo_ctx *c, int timestep) {
  if (!c) return FARGO_ERR_STATE;
  int rc;
  if ((rc = read_ctl(c))) return rc;
  const Ctl k = *c->pin_ctl;
  const DevParams &P = c->dp;
  const std::string dir = c->P.outputdir;
  const int L = FARGO_FORCE_LEVELS;
  for (int b = 0; b < k.nb; b++) {
    const double x = k.x[b], y = k.y[b], vx = k.vx[b], vy = k.vy[b], m = k.mass[b];
    const double r = sqrt(x * x + y * y), a = sqrt(x * x + y * y);
    const double rh = pow(m / 3., 1. / 3.) * a + 1e-15;
    const double sm = P.roche_smoothing ? r * pow(m / 3., 1. / 3.) * P.rochesmoothing
                                        : fargo_smoothing(P, r, k.PhysicalTime, k.PhysicalTimeInitial);
    double gf[4 * FARGO_FORCE_LEVELS];
    if ((rc = fargo_compute_force(c, x, y, sm, m, a, rh, gf))) return rc;
    const double fxi = gf[0], fxei = gf[L - 1], fxo = gf[L], fxeo = gf[2 * L - 1];
    const double fyi = gf[2 * L], fyei = gf[3 * L - 1], fyo = gf[3 * L], fyeo = gf[4 * L - 1];
    const double row[9] = {x * fyi - y * fxi,   x * fyo - y * fxo,   x * fyei - y * fxei,   x * fyeo - y * fxeo,
                           vx * fxi + vy * fyi, vx * fxo + vy * fyo, vx * fxei + vy * fyei, vx * fxeo + vy * fyeo,
                           k.PhysicalTime};
    if ((rc = host_append_row(dir, "tqwk" + std::to_string(b) + ".dat", timestep, row, 9)))
      return set_err(c, rc, "cannot write tqwk file");
    if (c->P.self_gravity) continue;
    for (int l = 0; l < L; l++) {
      const double lr[5] = {x * gf[2 * L + l] - y * gf[l], x * gf[3 * L + l] - y * gf[L + l],
                            vx * gf[l] + vy * gf[2 * L + l], vx * gf[L + l] + vy * gf[3 * L + l], k.PhysicalTime};
      if ((rc = host_append_row(dir, "tqwk" + std::to_string(b) + "_" + std::to_string(l) + ".dat", timestep, lr, 5)))
        return set_err(c, rc, "cannot write tqwk file");
    }
  }
  return FARGO_OK;
}

int fargo_restart(fargo_ctx *c, int index) {
  if (!c) return FARGO_ERR_STATE;
  if (index < 0) return set_err(c, FARGO_ERR_INVALID, "negative restart index");
  const fargo_params &p = c->P;
  const std::string dir = p.outputdir;
  const size_t n = c->h.size_grid, nout = (size_t)p.nrad * p.nsec;
  const char *names[4] = {"dens", "vrad", "vtheta", "energy"};
  const int which[4] = {FARGO_FIELD_DENS, FARGO_FIELD_VRAD, FARGO_FIELD_VTHETA, FARGO_FIELD_ENERGY};
  std::vector<double> f[4];
  int rc;
  for (int q = 0; q < 4; q++) {
    if (q == 3 && !p.adiabatic) continue;
    f[q].resize(n);
    if ((rc = fargo_get_field(c, which[q], f[q].data()))) return rc;  // ring nrad: the created context's
    if ((rc = host_read_field(dir, names[q], index, f[q].data(), nout)))
      return set_err(c, rc, std::string("cannot read ") + names[q] + std::to_string(index) + ".dat");
  }
  if ((rc = fargo_set_fields(c, f[0].data(), f[1].data(), f[2].data(), p.adiabatic ? f[3].data() : nullptr)))
    return rc;
  if ((rc = read_ctl(c))) return rc;
  Ctl &k = *c->pin_ctl;
  double lost = 0.0, t = (double)index * p.ninterm * p.dt, omega = k.OmegaFrame;
  for (int b = 0; b < k.nb; b++) {
    fargo_planet pl{};
    if ((rc = host_read_planet_row(dir, b, index, pl, &lost, &t, &omega)))
      return set_err(c, rc, "cannot read row " + std::to_string(index) + " of planet" + std::to_string(b) + ".dat");
    k.x[b] = pl.x;
    k.y[b] = pl.y;
    k.vx[b] = pl.vx;
    k.vy[b] = pl.vy;
    k.mass[b] = pl.mass;
  }
  k.PhysicalTime = t;
  k.OmegaFrame = omega;
  k.LostMass = lost;
  fargo_planet_params(k, c->dp, k.PhysicalTime);
  if ((rc = write_ctl(c))) return rc;
  for (int b = 0; b < k.nb; b++)
    if ((rc = host_truncate_planet_file(dir, b, index))) return set_err(c, rc, "cannot rewrite planet file");
  return FARGO_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Fused ensembles.  Every disk keeps its own context (fields, control block, ring
// tables); the plan gathers their kernel arguments in one device array and, for
// each substep kernel, one launch group: the members that run it, each member's
// own grid (the single-disk launch's), one block size (the largest member's, for
// the kernels whose block follows the ring width) and shared memory (the largest).
// One graph per DT round: the DT start of every disk, then a conditional while
// node whose body is one substep of every disk not yet done.  A disk is done when
// its own DT is (k_end's test, src/SourceEuler.cu:222); its blocks then return at
// once, and the loop ends with the last disk.  Each disk runs the single-disk
// kernel bodies in the single-disk order, so its results are bitwise those of the
// disk run alone.
struct fargo_fused {
  int precision = FARGO_FP64;
  int n = 0;
  int lanes = 1;
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<void *> bufs;  // device: arguments, control-block table, group tables
  int per_substep = 0, per_dt = 0;
  // the launches of the plan, for fused_time_kernels: the DT start, then the
  // substep groups (lane by lane)
  struct Launch {
    const char *name;
    std::function<void(cudaStream_t, int)> fn;  // (stream, programmatic launch)
  };
  std::vector<Launch> head, body;
  std::vector<std::string> names;  // of the last fused_time_kernels
};

namespace {
struct FusedGroup {
  int kernel;
  std::vector<int> member, first, gx, gy;  // first: prefix sums of the launched blocks
  dim3 block;
  size_t smem = 0;
  int extra = 0;
  int merge = 1;  // consecutive blocks of a disk's grid along x per launched block
};
// launched blocks of the per-cell kernels cover this many blocks of their disk
constexpr int FUSED_CELL_MERGE = 4;

const char *batch_kernel_name(int k) {
  static const char *const names[BK_END + 1] = {
      "kb_dt_begin", "kb_soundspeed", "kb_cfl_forces (4 cells/thread)", "kb_cfl_forces", "kb_planets",
      "kb_correct_vtheta", "kb_source", "kb_visc_tau", "kb_visc_update", "kb_artvisc", "kb_energy", "kb_radial",
      "kb_radial_col", "kb_azimuthal4", "kb_azimuthal4 (chunks/thread)", "kb_velocities", "kb_end"};
  return k >= 0 && k <= BK_END ? names[k] : "?";
}

template <class T>
int fused_build(fargo_fused *f, fargo_ctx *const *disks, int n, int by_width, std::string *why) {
  std::vector<KArgs<T>> args(n);
  size_t az_smem_all = 0;
  for (int k = 0; k < n; k++) {
    const fargo_ctx *c = disks[k];
    const fargo_params &p = c->P;
    const char *no = p.self_gravity ? "self-gravity"
                   : (p.open_inner || p.non_reflecting || p.evanescent) ? "an open, non-reflecting or evanescent boundary"
                   : p.sloppy_cfl ? "the sloppy CFL (-c)"
                   : !c->az_regs ? "a ring too wide for the register azimuthal sweep"
                   : nullptr;
    if (no) {
      *why = "disk " + std::to_string(k) + " uses " + no + ", which the fused form does not carry";
      return FARGO_ERR_INVALID;
    }
    KArgs<T> a = make_args<T>(c);
    a.use_cond = 0;
    a.guard = 0;
    a.mode = 0;
    a.pdl = 1;
    a.rad_maps = nullptr;
    a.cell_bx = 64;
    a.cell_by = 4;
    args[k] = a;
    az_smem_all = std::max(az_smem_all, c->az_smem);
  }
  auto dev = [&](const void *src, size_t bytes) -> void * {
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    f->bufs.push_back(p);
    if (cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return nullptr;
    return p;
  };
  const KArgs<T> *args_dev = (const KArgs<T> *)dev(args.data(), n * sizeof(KArgs<T>));
  std::vector<Ctl *> ctls(n);
  for (int k = 0; k < n; k++) ctls[k] = disks[k]->d_ctl;
  Ctl *const *ctls_dev = (Ctl *const *)dev(ctls.data(), n * sizeof(Ctl *));
  if (!args_dev || !ctls_dev) {
    *why = "device allocation of the fused plan failed";
    return FARGO_ERR_CUDA;
  }
  // lanes: one per ring width (by_width), or one for every disk.  Width 0 = any.
  std::vector<int> widths;
  if (by_width) {
    for (int k = 0; k < n; k++) widths.push_back(disks[k]->P.nsec);
    std::sort(widths.begin(), widths.end());
    widths.erase(std::unique(widths.begin(), widths.end()), widths.end());
  } else {
    widths.push_back(0);
  }
  // launch groups in substep order
  auto group = [&](int kernel, int width, auto pred, auto grid, dim3 block, size_t smem, int extra, int merge = 1) {
    FusedGroup g;
    g.kernel = kernel;
    g.block = block;
    g.smem = smem;
    g.extra = extra;
    g.merge = merge;
    g.first.push_back(0);
    for (int k = 0; k < n; k++) {
      if (width && disks[k]->P.nsec != width) continue;
      if (!pred(disks[k]->P, disks[k])) continue;
      const int2 gd = grid(disks[k]->P, disks[k]);
      g.member.push_back(k);
      g.gx.push_back(gd.x);
      g.gy.push_back(gd.y);
      g.first.push_back(g.first.back() + (gd.x + merge - 1) / merge * gd.y);
    }
    return g;
  };
  auto all = [](const fargo_params &, const fargo_ctx *) { return true; };
  auto one = [](const fargo_params &, const fargo_ctx *) { return make_int2(1, 1); };
  auto rings = [](const fargo_params &p, const fargo_ctx *) { return make_int2(p.nrad, 1); };
  auto cells = [](const fargo_params &p, const fargo_ctx *) { return make_int2((p.nsec + 63) / 64, (p.nrad + 3) / 4); };
  auto tiles = [](const fargo_params &p, const fargo_ctx *) {
    return make_int2((p.nsec + 31) / 32, (p.nrad + RAD_TR - 1) / RAD_TR);
  };
  auto columns = [](const fargo_params &p, const fargo_ctx *) {
    return make_int2((p.nsec + RADC_THREADS - 1) / RADC_THREADS, (p.nrad + RADC_RINGS - 1) / RADC_RINGS);
  };
  auto rad_col = [](const fargo_params &, const fargo_ctx *c) { return c->rad_col; };
  auto rad_tile = [](const fargo_params &, const fargo_ctx *c) { return !c->rad_col; };
  auto v4 = [](const fargo_params &p, const fargo_ctx *) { return p.nsec % 4 == 0 && p.nsec >= 260 && p.nsec <= 1024; };
  auto not_v4 = [&](const fargo_params &p, const fargo_ctx *c) { return !v4(p, c); };
  auto adiabatic = [](const fargo_params &p, const fargo_ctx *) { return p.adiabatic != 0; };
  auto corot = [](const fargo_params &p, const fargo_ctx *) { return p.corotating != 0; };
  auto az_mc = [](const fargo_params &p, const fargo_ctx *) { return p.nsec / 4 > az4_threads_host<T>(p.nsec); };
  auto az_one = [&](const fargo_params &p, const fargo_ctx *c) { return !az_mc(p, c); };
  const dim3 b2(64, 4);
  std::vector<FusedGroup> head = {group(BK_DT_BEGIN, 0, all, one, dim3(32), 0, 0),
                                  group(BK_SOUNDSPEED, 0, adiabatic, rings, dim3(256), 0, 0)};
  std::vector<std::vector<FusedGroup>> body;  // per lane
  for (const int w : widths) {
    // the blocks that follow the ring width take the lane's widest member
    int v4_threads = 32, az_threads = 32;
    size_t az_smem = 0;
    for (int k = 0; k < n; k++) {
      const fargo_params &p = disks[k]->P;
      if (w && p.nsec != w) continue;
      if (v4(p, disks[k])) v4_threads = std::max(v4_threads, (p.nsec / 4 + 31) / 32 * 32);
      az_threads = std::max(az_threads, az4_threads_host<T>(p.nsec));
      az_smem = std::max(az_smem, disks[k]->az_smem);
    }
    body.push_back({group(BK_CFL_V4, w, v4, rings, dim3(v4_threads), 0, 0),
                    group(BK_CFL, w, not_v4, rings, dim3(256), 0, 0),
                    group(BK_PLANETS, w, all, one, dim3(64), 0, 0),
                    group(BK_COROT, w, corot, cells, b2, 0, 0, FUSED_CELL_MERGE),
                    group(BK_SOURCE, w, all, cells, b2, 0, 0, FUSED_CELL_MERGE),
                    group(BK_VISC_TAU, w, all, cells, b2, 0, 0, FUSED_CELL_MERGE),
                    group(BK_VISC_UPDATE, w, all, cells, b2, 0, 0, FUSED_CELL_MERGE),
                    group(BK_ARTVISC, w, all, cells, b2, 0, 0, FUSED_CELL_MERGE),
                    group(BK_ENERGY, w, adiabatic, cells, b2, 0, 0, FUSED_CELL_MERGE),
                    group(BK_RADIAL, w, rad_tile, tiles, dim3(32, RAD_NY_HOST), rad_smem_bytes(sizeof(T)), 0),
                    group(BK_RADIAL_COL, w, rad_col, columns, dim3(RADC_THREADS), 0, 0),
                    group(BK_AZ4, w, az_one, rings, dim3(az_threads), az_smem, 0),
                    group(BK_AZ4_MC, w, az_mc, rings, dim3(sizeof(T) == 8 ? 512 : 768), az_smem, 0),
                    group(BK_VELOCITIES, w, all, cells, b2, 0, 1, FUSED_CELL_MERGE),
                    group(BK_END, w, all, one, dim3(256), 0, 0)});
  }
  if (prepare_batched<T>(rad_smem_bytes(sizeof(T)), az_smem_all) != cudaSuccess) {
    *why = "cudaFuncSetAttribute on the batched kernels failed";
    return FARGO_ERR_CUDA;
  }
  auto to_dev = [&](const FusedGroup &g, BatchGroup<T> &G) -> bool {
    G.args = args_dev;
    G.ng = (int)g.member.size();
    G.extra = g.extra;
    std::vector<int4> blk;
    blk.reserve(g.first.back());
    for (size_t m = 0; m < g.member.size(); m++) {
      const int gx = g.gx[m], gy = g.gy[m], nb = gx * gy;
      for (int by = 0; by < gy; by++)
        for (int bx = 0; bx < gx; bx += g.merge) {
          const int cnt = std::min(g.merge, gx - bx);
          blk.push_back(make_int4(g.member[m] | (cnt << 20), bx, by, nb));
        }
    }
    G.blk = (const int4 *)dev(blk.data(), blk.size() * sizeof(int4));
    return G.blk != nullptr;
  };
  auto add = [&](std::vector<fargo_fused::Launch> &to, const FusedGroup &g) -> bool {
    if (g.member.empty()) return true;
    BatchGroup<T> G;
    if (!to_dev(g, G)) return false;
    const int kernel = g.kernel, nb = g.first.back();
    const dim3 block = g.block;
    const size_t smem = g.smem;
    to.push_back({batch_kernel_name(kernel),
                  [=](cudaStream_t s, int pdl) { launch_batched<T>(kernel, G, nb, block, smem, pdl, s); }});
    return true;
  };
  for (const FusedGroup &g : head)
    if (!add(f->head, g)) return FARGO_ERR_CUDA;
  std::vector<size_t> lane_end;  // f->body index after each lane
  for (const auto &lane : body) {
    for (const FusedGroup &g : lane)
      if (!add(f->body, g)) return FARGO_ERR_CUDA;
    lane_end.push_back(f->body.size());
  }
  f->lanes = (int)body.size();
  if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess) return FARGO_ERR_CUDA;
  // the graph: the DT start of every disk, then the while loop of substeps
  cudaGraph_t g = nullptr, gp = nullptr;
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return FARGO_ERR_CUDA;
  f->graph = g;
  LaunchProbe probe;
  std::memset(&probe, 0, sizeof(probe));
  g_probe = &probe;
  if (cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return FARGO_ERR_CUDA;
  for (const auto &l : f->head) l.fn(f->stream, 1);
  g_probe = nullptr;
  if (cudaStreamEndCapture(f->stream, &gp) != cudaSuccess) return FARGO_ERR_CUDA;
  f->per_dt = probe.count;
  cudaGraphNode_t np, nc;
  if (cudaGraphAddChildGraphNode(&np, g, nullptr, 0, gp) != cudaSuccess) return FARGO_ERR_CUDA;
  cudaGraphDestroy(gp);
  cudaGraphConditionalHandle h;
  if (cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) return FARGO_ERR_CUDA;
  cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  if (cudaGraphAddNode(&nc, g, &np, nullptr, 1, &cp) != cudaSuccess) return FARGO_ERR_CUDA;
  cudaGraph_t loop = cp.conditional.phGraph_out[0];
  // the loop body: each lane's substep on a stream of its own (lane 0 on the plan's
  // stream), forked from and joined back into the plan's stream; every lane's first
  // launch and the loop condition after the join are plain launches
  const int L = f->lanes;
  std::vector<cudaStream_t> ls(L, f->stream);
  std::vector<cudaEvent_t> ev(L, nullptr);
  bool ok = true;
  for (int l = 0; l < L && ok; l++) {
    ok = cudaEventCreateWithFlags(&ev[l], cudaEventDisableTiming) == cudaSuccess;
    if (ok && l > 0) ok = cudaStreamCreateWithFlags(&ls[l], cudaStreamNonBlocking) == cudaSuccess;
  }
  auto cleanup = [&]() {
    for (int l = 0; l < L; l++) {
      if (ev[l]) cudaEventDestroy(ev[l]);
      if (l > 0 && ls[l] != f->stream && ls[l]) cudaStreamDestroy(ls[l]);
    }
  };
  if (!ok) {
    cleanup();
    return FARGO_ERR_CUDA;
  }
  if (cudaStreamBeginCaptureToGraph(f->stream, loop, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
      cudaSuccess) {
    cleanup();
    return FARGO_ERR_CUDA;
  }
  probe.count = 0;
  g_probe = &probe;
  if (L > 1) {
    cudaEventRecord(ev[0], f->stream);
    for (int l = 1; l < L; l++) cudaStreamWaitEvent(ls[l], ev[0], 0);
  }
  for (int l = 0; l < L; l++) {
    const size_t b0 = l ? lane_end[l - 1] : 0;
    for (size_t q = b0; q < lane_end[l]; q++) f->body[q].fn(ls[l], L > 1 && q == b0 ? 0 : 1);
  }
  for (int l = 1; l < L; l++) {
    cudaEventRecord(ev[l], ls[l]);
    cudaStreamWaitEvent(f->stream, ev[l], 0);
  }
  launch_loop_cond(ctls_dev, n, (unsigned long long)h, L > 1 ? 0 : 1, f->stream);
  g_probe = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(f->stream, &loop);
  cleanup();
  if (ce != cudaSuccess) return FARGO_ERR_CUDA;
  f->per_substep = probe.count;
  if (cudaGraphInstantiate(&f->exec, g, 0) != cudaSuccess) return FARGO_ERR_CUDA;
  return FARGO_OK;
}
}  // namespace

int fused_create(fargo_ctx *const *disks, int n, int by_width, fargo_fused **out, std::string *why) {
  *out = nullptr;
  if (!disks || n <= 0 || n >= (1 << 20)) return FARGO_ERR_INVALID;  // disk index: 20 bits of a table entry
  for (int k = 0; k < n; k++)
    if (disks[k]->precision != disks[0]->precision) {
      *why = "the disks of a fused ensemble share one precision";
      return FARGO_ERR_INVALID;
    }
  // every disk's own queue is drained first: the plan reads their control blocks
  for (int k = 0; k < n; k++)
    if (cudaStreamSynchronize(disks[k]->stream) != cudaSuccess) return FARGO_ERR_CUDA;
  fargo_fused *f = new fargo_fused();
  f->precision = disks[0]->precision;
  f->n = n;
  const int rc = f->precision == FARGO_FP64 ? fused_build<double>(f, disks, n, by_width, why)
                                             : fused_build<float>(f, disks, n, by_width, why);
  if (rc != FARGO_OK) {
    if (why->empty()) *why = std::string("building the fused plan: ") + cudaGetErrorString(cudaGetLastError());
    fused_destroy(f);
    return rc;
  }
  *out = f;
  return FARGO_OK;
}

int fused_run(fargo_fused *f, int ndt) {
  for (int k = 0; k < ndt; k++)
    if (cudaGraphLaunch(f->exec, f->stream) != cudaSuccess) return FARGO_ERR_CUDA;
  return FARGO_OK;
}

int fused_sync(fargo_fused *f) { return cudaStreamSynchronize(f->stream) == cudaSuccess ? FARGO_OK : FARGO_ERR_CUDA; }

int fused_launches(const fargo_fused *f, int *per_substep, int *per_dt) {
  if (per_substep) *per_substep = f->per_substep;
  if (per_dt) *per_dt = f->per_dt;
  return FARGO_OK;
}

int fused_lanes(const fargo_fused *f) { return f->lanes; }

int fused_time_kernels(fargo_fused *f, int reps, double *ms, int cap, int *ngroups) {
  if (reps <= 0 || !ms || !ngroups) return FARGO_ERR_INVALID;
  const int G = (int)f->body.size();
  if (cap < G) return FARGO_ERR_INVALID;
  if (cudaStreamSynchronize(f->stream) != cudaSuccess) return FARGO_ERR_CUDA;
  std::vector<cudaEvent_t> ev(G + 1, nullptr);
  for (auto &e : ev)
    if (cudaEventCreate(&e) != cudaSuccess) {
      for (auto &x : ev)
        if (x) cudaEventDestroy(x);
      return FARGO_ERR_CUDA;
    }
  for (const auto &l : f->head) l.fn(f->stream, 0);
  std::vector<double> acc(G, 0.0);
  int rc = FARGO_OK;
  for (int r = 0; r < reps && rc == FARGO_OK; r++) {
    cudaEventRecord(ev[0], f->stream);
    for (int q = 0; q < G; q++) {
      f->body[q].fn(f->stream, 0);
      cudaEventRecord(ev[q + 1], f->stream);
    }
    if (cudaStreamSynchronize(f->stream) != cudaSuccess) rc = FARGO_ERR_CUDA;
    for (int q = 0; q < G && rc == FARGO_OK; q++) {
      float t = 0.0f;
      cudaEventElapsedTime(&t, ev[q], ev[q + 1]);
      acc[q] += t;
    }
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if (rc != FARGO_OK) return rc;
  f->names.clear();
  for (int q = 0; q < G; q++) {
    ms[q] = acc[q] / reps;
    f->names.push_back(f->body[q].name);
  }
  *ngroups = G;
  return FARGO_OK;
}

const char *fused_kernel_name(const fargo_fused *f, int k) {
  return k >= 0 && k < (int)f->names.size() ? f->names[k].c_str() : nullptr;
}

void fused_destroy(fargo_fused *f) {
  if (!f) return;
  if (f->stream) cudaStreamSynchronize(f->stream);
  if (f->exec) cudaGraphExecDestroy(f->exec);
  if (f->graph) cudaGraphDestroy(f->graph);
  for (void *p : f->bufs) cudaFree(p);
  if (f->stream) cudaStreamDestroy(f->stream);
  delete f;
}
