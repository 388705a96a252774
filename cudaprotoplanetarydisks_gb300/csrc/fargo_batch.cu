// fargo_batch.cu -- an ensemble of independent disks advanced together.
//
// Every disk is a context of its own (fargo_ctx: fields, one DT graph with the
// CFL loop on the device, its own streams), so every disk keeps its own CFL step
// and substep count.  The batch enqueues the disks' DT graphs round-robin on their
// streams and synchronises once: the GPU runs the graphs of many disks at the same
// time, which fills the SMs that one small disk leaves idle (a 128x384 disk's
// kernels are one partial wave each).  Nothing is shared between disks but the
// device, so a disk's results are bitwise those of the same disk run alone.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <vector>

#include <cuda_runtime.h>

#include <string>

#include "fargo_gb300.h"
#include "fargo_internal.h"

struct fargo_batch {
  std::vector<fargo_ctx *> disks;
  std::vector<double> dt;           // DT of each disk (its parameter file's DT)
  fargo_fused *fused = nullptr;     // the fused form (fargo_batch_fuse), or none
  std::string err;
};

extern "C" {

int fargo_batch_create(int n, const fargo_params *params, const fargo_planet *planets, const int *nplanets,
                       int precision, fargo_batch **out) {
  return fargo_batch_create_variant(n, params, planets, nplanets, precision, nullptr, out);
}

int fargo_batch_create_variant(int n, const fargo_params *params, const fargo_planet *planets,
                               const int *nplanets, int precision, const fargo_variant *v, fargo_batch **out) {
  if (!out || n <= 0 || !params || !nplanets) return FARGO_ERR_INVALID;
  *out = nullptr;
  fargo_batch *b = new fargo_batch();
  int off = 0;
  for (int k = 0; k < n; k++) {
    if (nplanets[k] < 0 || (nplanets[k] > 0 && !planets)) {
      fargo_batch_destroy(b);
      return FARGO_ERR_INVALID;
    }
    fargo_ctx *c = nullptr;
    const int rc = fargo_ctx_create_variant(&params[k], nplanets[k] ? planets + off : nullptr, nplanets[k],
                                            precision, nullptr, v, &c);
    if (rc != FARGO_OK) {
      fargo_batch_destroy(b);
      return rc;
    }
    b->disks.push_back(c);
    b->dt.push_back(params[k].dt);
    off += nplanets[k];
  }
  *out = b;
  return FARGO_OK;
}

void fargo_batch_destroy(fargo_batch *b) {
  if (!b) return;
  fused_destroy(b->fused);
  for (fargo_ctx *c : b->disks) fargo_ctx_destroy(c);
  delete b;
}

int fargo_batch_size(const fargo_batch *b) { return b ? (int)b->disks.size() : 0; }

fargo_ctx *fargo_batch_disk(fargo_batch *b, int k) {
  if (!b || k < 0 || k >= (int)b->disks.size()) return nullptr;
  return b->disks[k];
}

// ndt[k] DTs on disk k (ndt == NULL: ndt_all on every disk), enqueued round-robin
// (DT 1 of every disk, then DT 2, ...) so that every stream has work at once.
static int enqueue(fargo_batch *b, const int *ndt, int ndt_all) {
  int most = 0;
  for (size_t k = 0; k < b->disks.size(); k++) most = std::max(most, ndt ? ndt[k] : ndt_all);
  for (int d = 0; d < most; d++)
    for (size_t k = 0; k < b->disks.size(); k++)
      if (d < (ndt ? ndt[k] : ndt_all)) {
        const int rc = fargo_run_async(b->disks[k], 1);
        if (rc != FARGO_OK) return rc;
      }
  return FARGO_OK;
}

int fargo_batch_run_async(fargo_batch *b, int ndt) {
  if (!b || ndt < 0) return FARGO_ERR_STATE;
  if (b->fused) return fused_run(b->fused, ndt);
  return enqueue(b, nullptr, ndt);
}

int fargo_batch_fuse_by_width(fargo_batch *b, int by_width) {
  if (!b) return FARGO_ERR_STATE;
  by_width = by_width ? 1 : 0;
  if (b->fused && (fused_lanes(b->fused) > 1) == (by_width == 1)) return FARGO_OK;
  if (b->fused) {
    const int rc = fused_sync(b->fused);
    fused_destroy(b->fused);
    b->fused = nullptr;
    if (rc != FARGO_OK) return rc;
  }
  b->err.clear();
  return fused_create(b->disks.data(), (int)b->disks.size(), by_width, &b->fused, &b->err);
}

int fargo_batch_fuse(fargo_batch *b) { return fargo_batch_fuse_by_width(b, 1); }

int fargo_batch_fused_lanes(const fargo_batch *b, int *lanes) {
  if (!b || !b->fused || !lanes) return FARGO_ERR_STATE;
  *lanes = fused_lanes(b->fused);
  return FARGO_OK;
}

int fargo_batch_fused_time_kernels(fargo_batch *b, int reps, double *ms_per_group, int cap, int *ngroups) {
  if (!b || !b->fused) return FARGO_ERR_STATE;
  return fused_time_kernels(b->fused, reps, ms_per_group, cap, ngroups);
}

const char *fargo_batch_fused_kernel_name(const fargo_batch *b, int k) {
  return b && b->fused ? fused_kernel_name(b->fused, k) : nullptr;
}

const char *fargo_batch_last_error(const fargo_batch *b) { return b ? b->err.c_str() : ""; }

int fargo_batch_fused_launches(const fargo_batch *b, int *per_substep, int *per_dt) {
  if (!b || !b->fused) return FARGO_ERR_STATE;
  return fused_launches(b->fused, per_substep, per_dt);
}

int fargo_batch_sync(fargo_batch *b) {
  if (!b) return FARGO_ERR_STATE;
  if (b->fused) {
    const int rc = fused_sync(b->fused);
    if (rc != FARGO_OK) return rc;
  }
  for (fargo_ctx *c : b->disks) {
    const int rc = fargo_sync(c);
    if (rc != FARGO_OK) return rc;
  }
  return FARGO_OK;
}

// Every disk advances whole DTs (its own DT) until its physical time reaches t_end
// (within 1e-9 of a DT); substeps of all disks are summed into *nsub.  A disk
// whose device flags an error makes the call return that disk's status (its
// message: fargo_last_error of fargo_batch_disk(b, k)); *failed = that k or -1.
int fargo_batch_advance(fargo_batch *b, double t_end, long long *nsub, int *failed) {
  if (failed) *failed = -1;
  if (!b) return FARGO_ERR_STATE;
  const size_t n = b->disks.size();
  std::vector<int> ndt(n, 0);
  std::vector<long long> s0(n, 0);
  for (size_t k = 0; k < n; k++) {
    fargo_scalars s;
    int rc = fargo_get_scalars(b->disks[k], &s);
    if (rc != FARGO_OK) return rc;
    s0[k] = s.substeps;
    const double left = (t_end - s.physical_time) / b->dt[k];
    ndt[k] = left > 1e-9 ? (int)std::ceil(left - 1e-9) : 0;
  }
  bool same = true;
  for (size_t k = 1; k < n; k++) same = same && ndt[k] == ndt[0];
  int rc = (b->fused && same) ? fused_run(b->fused, n ? ndt[0] : 0) : enqueue(b, ndt.data(), 0);
  if (rc == FARGO_OK && b->fused) rc = fused_sync(b->fused);
  if (rc != FARGO_OK) return rc;
  long long tot = 0;
  for (size_t k = 0; k < n; k++) {
    // fargo_run with no DT reads the control block and reports a device error
    long long sub = 0;
    rc = fargo_run(b->disks[k], 0, &sub);
    if (rc != FARGO_OK) {
      if (failed) *failed = (int)k;
      return rc;
    }
    fargo_scalars s;
    if ((rc = fargo_get_scalars(b->disks[k], &s)) != FARGO_OK) return rc;
    tot += s.substeps - s0[k];
  }
  if (nsub) *nsub = tot;
  return FARGO_OK;
}

// Cell updates per second of the disks in variant v: a fresh batch, one warm-up
// DT, then ndt DTs on every disk
static int batch_rate(int n, const fargo_params *params, const fargo_planet *planets, const int *nplanets,
                      int precision, const fargo_variant &v, int ndt, double *rate) {
  fargo_batch *b = nullptr;
  int rc = fargo_batch_create_variant(n, params, planets, nplanets, precision, &v, &b);
  if (rc != FARGO_OK) return rc;
  std::vector<long long> s0(n);
  if ((rc = fargo_batch_run_async(b, 1)) == FARGO_OK) rc = fargo_batch_sync(b);
  for (int k = 0; k < n && rc == FARGO_OK; k++) {
    fargo_scalars s;
    rc = fargo_get_scalars(b->disks[k], &s);
    s0[k] = s.substeps;
  }
  const auto t0 = std::chrono::steady_clock::now();
  if (rc == FARGO_OK && (rc = fargo_batch_run_async(b, ndt)) == FARGO_OK) rc = fargo_batch_sync(b);
  const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  double cells = 0.0;
  for (int k = 0; k < n && rc == FARGO_OK; k++) {
    fargo_scalars s;
    rc = fargo_get_scalars(b->disks[k], &s);
    cells += (double)(s.substeps - s0[k]) * params[k].nrad * params[k].nsec;
  }
  fargo_batch_destroy(b);
  if (rc == FARGO_OK) *rate = t > 0.0 ? cells / t : 0.0;
  return rc;
}

int fargo_batch_autotune(int n, const fargo_params *params, const fargo_planet *planets, const int *nplanets,
                         int precision, int ndt, fargo_variant *best, double *rate_best, double *rate_default) {
  if (!best || n <= 0 || !params || !nplanets || ndt < 1) return FARGO_ERR_INVALID;
  fargo_variant v;
  fargo_variant_default(&v);
  double r = 0.0;
  int rc = batch_rate(n, params, planets, nplanets, precision, v, ndt, &r);
  if (rc != FARGO_OK) return rc;
  if (rate_default) *rate_default = r;
  bool sg = false;
  for (int k = 0; k < n; k++) sg = sg || params[k].self_gravity;
  // one knob at a time: every other value of the knob on the best variant so far
  struct Knob {
    int fargo_variant::*field;
    int nvals;  // values 0 .. nvals - 1
    bool on;
  } knobs[] = {{&fargo_variant::pad, 2, true},
               {&fargo_variant::priority, 3, true},
               {&fargo_variant::sg_ahead, 2, sg},
               {&fargo_variant::pdl, 2, true},
               // tile and launch shapes: the per-cell kernels' CTA (64x4, 32x8, 128x2,
               // 256x1), the radial transport's TMA-staged persistent form and its
               // column march (the
               // azimuthal sweep's chunks per thread change the ring mean's summation
               // order, so that knob is not searched: every candidate here is bitwise
               // the default)
               {&fargo_variant::cell_block, 4, true},
               {&fargo_variant::rad_tma, 2, true},
               {&fargo_variant::rad_col, 2, true}};
  for (const Knob &kn : knobs) {
    if (!kn.on) continue;
    const fargo_variant base = v;
    for (int val = 0; val < kn.nvals; val++) {
      if (val == base.*kn.field) continue;
      fargo_variant cand = base;
      cand.*kn.field = val;
      double cr = 0.0;
      if ((rc = batch_rate(n, params, planets, nplanets, precision, cand, ndt, &cr)) != FARGO_OK) return rc;
      if (cr > r * 1.005) {
        r = cr;
        v = cand;
      }
    }
  }
  *best = v;
  if (rate_best) *rate_best = r;
  return FARGO_OK;
}

}  // extern "C"
