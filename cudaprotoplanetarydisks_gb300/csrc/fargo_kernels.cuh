// fargo_kernels.cuh -- launch interface of the step kernels (fargo_kernels.cu, fargo_sg.cu).
#pragma once

#include <cuda_runtime.h>

#include "fargo_device.cuh"

// parts of one substep, in launch order
#define SUBK_CFL_FORCES  0x001u  // ConditionCFL + ComputeAccel + FillForcesArrays (planets) + planets
#define SUBK_COROT       0x002u  // CorrectVtheta (corotating frame)
#define SUBK_BC1         0x004u  // ApplyBoundaryCondition before the source step
#define SUBK_SG          0x008u  // compute_selfgravity
#define SUBK_SOURCE      0x010u  // pressure, Substep1, viscosity, Substep2, host, Actualise
#define SUBK_BC2         0x020u  // ApplyBoundaryCondition after the source step
#define SUBK_ENERGY      0x040u  // ComputeViscousTerms + Substep3 (energy equation)
#define SUBK_TRANSPORT   0x080u  // Transport
#define SUBK_BC3         0x100u  // ApplyBoundaryCondition after transport
#define SUBK_TEMPERATURE 0x200u  // ComputeTemperatureField
#define SUBK_END         0x400u  // PhysicalTime, LostMass, loop condition
#define SUBK_ALL         0x7ffu

// Optional launch probe: counts launches and, when events are given, records one
// event after each kernel so the per-kernel device time can be read back.
struct LaunchProbe {
  cudaEvent_t ev[96];
  const char *name[96];
  int n;       // events recorded
  int count;   // launches seen
  int nev;     // events available (0: count only)
};
extern thread_local LaunchProbe *g_probe;
inline void probe_mark(cudaStream_t s, const char *name) {
  if (!g_probe) return;
  if (g_probe->n < g_probe->nev) {
    cudaEventRecord(g_probe->ev[g_probe->n], s);
    g_probe->name[g_probe->n] = name;
    g_probe->n++;
  }
  g_probe->count++;
}

// Kernel launch with the stream's priority as the launch's own (so that a graph
// captured from the stream keeps it per node), and the
// programmatic-stream-serialization attribute when pdl is set (the kernel begins
// with pdl_enter()).
template <typename... Exp, typename... Act>
inline void launch_k(int pdl, void (*kern)(Exp...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                     Act &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[2];
  int prio = 0;
  cudaStreamGetPriority(s, &prio);
  at[0].id = cudaLaunchAttributePriority;
  at[0].val.priority = prio;
  at[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl ? 2 : 1;
  cudaLaunchKernelEx(&cfg, kern, static_cast<Exp>(args)...);
}

void launch_convert_from_f64(const double *in, void *out, size_t n, int esize, cudaStream_t s);
void launch_convert_to_f64(const void *in, double *out, size_t n, int esize, cudaStream_t s);
// up to five fields converted in one launch: src[f] -> dst[f], n elements each
struct ConvFields {
  const void *src[5];
  void *dst[5];
  int nf;
};
void launch_convert_from_f64_multi(const ConvFields &p, size_t n, int esize, cudaStream_t s);
void launch_convert_to_f64_multi(const ConvFields &p, size_t n, int esize, cudaStream_t s);

// Second and third streams: the planet update of a substep runs beside the hydro
// kernels (forked after k_cfl_forces, joined at the end of the substep); the
// self-gravity transforms run beside k_cfl_forces.  Without them, or in a
// corotating frame (for the planets), everything runs in line.
struct SideBranch {
  cudaStream_t s;
  cudaEvent_t fork, join;
  // self-gravity beside the CFL/force kernel: both read the density at the start
  // of the substep and share no other data (used when no boundary kernel
  // changes the density in between)
  cudaStream_t s2;
  cudaEvent_t fork2, join2;
};

// DT loop rotation (the DT graph with self-gravity): a substep whose CFL/force
// kernel and self-gravity transforms ran ahead (ROT_HEAD_DONE) launches the next
// substep's after its k_end (ROT_NEXT_HEAD), guarded so that they do nothing once
// the DT is done; launch_dt_head runs the first substep's in the DT prefix.
#define ROT_HEAD_DONE 0x1u
#define ROT_NEXT_HEAD 0x2u
// Ring transforms ahead (the DT loop with self-gravity, not rotated): the
// azimuthal forward transforms of a substep's density ran before the substep (in
// the DT prefix, or at the end of the previous substep, beside its k_velocities
// and k_end, since the density is final after the azimuthal transport); the
// substep launches the next substep's after its own azimuthal transport.
#define SG_AHEAD 0x8u
template <class T>
void launch_substep_kernels(const KArgs<T> &a, cudaStream_t s, unsigned which_mask, size_t az_smem_bytes,
                            const SideBranch *side = nullptr, unsigned rot = 0);
template <class T>
void launch_dt_head(const KArgs<T> &a, cudaStream_t s, const SideBranch *side);
template <class T>
bool rotation_allowed(const KArgs<T> &a, const SideBranch *side);
template <class T>
bool sg_ahead_allowed(const KArgs<T> &a, const SideBranch *side);
template <class T>
void launch_dt_prefix(const KArgs<T> &a, cudaStream_t s);
template <class T>
void launch_cfl_only(const KArgs<T> &a, cudaStream_t s);
template <class T>
void launch_boundaries(const KArgs<T> &a, cudaStream_t s);
template <class T>
cudaError_t prepare_kernels(size_t az_smem_bytes, int az_regs);
// Fused ensembles: one launch of a substep kernel over a group of disks
// (fargo_kernels.cu, kb_*); the plan is built by fargo_fused.cu.
template <class T>
struct BatchGroup {
  const KArgs<T> *args;  // every disk's kernel arguments (device array, indexed by disk)
  const int4 *blk;       // [blocks of the launch] disk + (blocks covered << 20), the first block's x and
                         // y in the disk's own grid, the disk's blocks
  int ng;
  int extra;             // kb_visc_tau: 1 = the new velocities; kb_velocities: with temperature
};
enum BatchKernel {
  BK_DT_BEGIN, BK_SOUNDSPEED, BK_CFL_V4, BK_CFL, BK_PLANETS, BK_COROT, BK_SOURCE, BK_VISC_TAU,
  BK_VISC_UPDATE, BK_ARTVISC, BK_ENERGY, BK_RADIAL, BK_RADIAL_COL, BK_AZ4, BK_AZ4_MC, BK_VELOCITIES, BK_END
};
// column-march radial transport: threads (sectors) per CTA, rings per thread
#define RADC_THREADS 128
#define RADC_RINGS 32
template <class T>
void launch_batched(int kernel, const BatchGroup<T> &G, int nblocks, dim3 block, size_t smem, int pdl,
                    cudaStream_t s);
void launch_loop_cond(Ctl *const *ctls, int n, unsigned long long handle, int pdl, cudaStream_t s);
template <class T>
cudaError_t prepare_batched(size_t rad_smem, size_t az_smem);
template <class T>
int az4_threads_host(int nsec);
#define RAD_NY_HOST 10
size_t rad_smem_bytes(int esize);
// CTAs of the persistent TMA radial transport on this device (0: not launchable)
template <class T>
int rad_tma_grid(int nrad, int nsec);
// TMA box of the radial transport's staged tiles: sectors (33 rounded up to 16
// bytes) x rings (the tile's RAD_TR rings, two below, three above)
#define RAD_TR 16
#define RAD_BW(T) (sizeof(T) == 4 ? 36 : 34)
#define RAD_BR (RAD_TR + 5)

// self-gravity (fargo_sg.cu)
template <class T>
void launch_selfgravity(const KArgs<T> &a, cudaStream_t s);
template <class T>
void launch_sg_rows_fwd(const KArgs<T> &a, cudaStream_t s);
template <class T>
void launch_sg_cols_inv(const KArgs<T> &a, cudaStream_t s);
template <class T>
void launch_sg_kernel_spectra(const KArgs<T> &a, cudaStream_t s);
template <class T>
cudaError_t prepare_sg_kernels(int nsec, int n0);
int sg_radices(int n, int *rad);  // radix-4/2/3 plan; returns stage count, -1 if n has other factors
