#!/usr/bin/env python
"""Benchmark of the FARGO-ADSG hydro step on GB300.

Workload (default): the self-gravitating disk, 256 x 768 log grid on
[0.4, 4.0], Sigma ~ 1/r with disk mass 0.02, alpha = 1e-3, self-gravity through a
2*Nrad zero-padded log-r FFT convolution (softening 0.3 h), one migrating
planet q = 5e-4 from r = 1.5 with the indirect term, 1e-3 seeded noise
(cudaprotoplanetarydisks_gb300/configs/c2_selfgravity.par).  A step is one DT
(AlgoGas: CFL-subcycled hydro substeps); the metric counts cell updates,
Nrad * Nsec per hydro substep.

Own arm: the state stays in HBM; each timed step is one graph launch of a DT
(CFL loop on the device), timed with CUDA events on the launching stream, with an
L2 flush (a 256 MiB write) before every timed step.  The headline is the
FP32-bulk mode; the FP64 mode is measured in the same run, and the FP32 fields
are compared with the FP64 oracle after the same steps.  e2e: the same metric
through the C-ABI with host buffers (pinned FP64 arrays copied in and out every
step).

--impl reference: the reference has no CPU implementation of this path (every
substep is a CUDA kernel); its CPU restatement (the oracle, OpenMP over rings)
is timed on all host cores.

--gpus N (torchrun, one rank per GPU): replicas only -- every rank advances its
own disk; value = all ranks' cell updates / the slowest rank's time.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s"
L2_FLUSH_BYTES = 256 << 20
REF_BUDGET_S = 90.0  # time budget of the CPU reference arm's timed sample


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c2")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-ensemble measurement")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-correction measurement")
    ap.add_argument("--profile", choices=["fp32", "fp64"], default=None,
                    help="profiling target: warm-up DTs, then --steps substeps launched kernel by kernel "
                         "(kernels inside the DT graph's while loop are invisible to ncu)")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def reduce_over_ranks(ms, nsub):
    """Replicas only: the job's time is the slowest rank's and its work every
    rank's.  (max of ms, sum of nsub) over the ranks of the default process group
    (nccl: CUDA tensors; gloo: CPU tensors); the inputs alone without one."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms), float(nsub)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(ms)], dtype=torch.float64, device=dev)
    n = torch.tensor([float(nsub)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(n, op=dist.ReduceOp.SUM)
    return float(t.item()), float(n.item())


def job_value(nsub_all, cells, ms_max):
    """Whole-job cell-updates/s: every rank's cell updates over the slowest time."""
    return nsub_all * cells / (ms_max * 1e-3)


def workload(cfg):
    import cudaprotoplanetarydisks_gb300 as fg
    params, planets = fg.load_config(cfg)
    name = {"c1": "isothermal disk 128x384, 1 planet (fixed orbit)",
            "c2": "self-gravitating disk 256x768, alpha viscosity, migrating planet",
            "c3": "adiabatic disk with cooling 1024x3072, 1 planet",
            "wide": "adiabatic disk 2048x4096, non-reflecting inner boundary, guiding-center frame, "
                    "Jupiter-mass planet"}.get(cfg, cfg)
    return params, planets, name


def config_obj(params, name, cfg, extra=None):
    c = {"workload": name, "config_file": f"configs/{cfg}", "nrad": params.nrad, "nsec": params.nsec,
         "cells": params.nrad * params.nsec, "self_gravity": bool(params.self_gravity),
         "adiabatic": bool(params.adiabatic), "DT": params.dt, "step": "one DT (AlgoGas, CFL-subcycled)",
         "l2": "flushed (256 MiB write) before every timed step"}
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            f = tempfile.NamedTemporaryFile(prefix="clocks", suffix=".csv", delete=False)
            self.path = f.name
            f.close()
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the timed region starts once the sampler has written its first line
        t0 = time.time()
        while time.time() - t0 < 5.0:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path).read().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ---------------------------------------------------------------------------
# algorithmic bytes per launch (compulsory reads + writes of each kernel)
def kernel_bytes(name, params, esize):
    G = params.nrad * params.nsec
    ad = 1 if params.adiabatic else 0
    sg = 1 if params.self_gravity else 0
    M = params.nsec // 2 + 1
    spec = 2 * M * params.nrad * 16          # both work spectra, complex FP64
    khat = 2 * M * 2 * params.nrad * 16      # both kernel spectra
    fields = {
        "k_cfl_forces": (3 + ad) + (1 if True else 0),
        "k_source": (4 + ad + 2 * sg) + 3,
        "k_visc_tau": 3 + 4,
        "k_visc_update": 6 + 2,
        "k_artvisc": (3 + ad) + (2 + ad),
        "k_energy": 8 + 2,
        "k_transport_radial": (3 + ad) + (5 + ad),
        "k_transport_azimuthal": (6 + ad) + (5 + ad),
        "k_velocities": (5 + 1) + 3,
        "k_temperature": 3,
    }
    if name in fields:
        return fields[name] * G * esize
    if name == "k_sg_rows_fwd":
        return G * esize + spec
    if name == "k_sg_cols":
        return spec + khat + spec
    if name == "k_sg_rows_inv":
        return spec + G * esize + 2 * G * esize
    return 0


def ncu_traffic(kernel, cfg, mode="fp32"):
    """DRAM bytes (read + write) of one launch of `kernel` from the committed ncu
    summary profiles/kernels_<cfg>_<mode>.md (one cold-cache capture), or None."""
    path = os.path.join(ROOT, "profiles", f"kernels_{cfg}_{mode}.md")
    if not os.path.exists(path):
        return None
    scale = {"B": 1.0, "KB": 1e3, "MB": 1e6, "GB": 1e9}
    for line in open(path):
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cells) >= 4 and cells[0] == kernel:
            try:
                rd, ru = cells[2].split()
                wr, wu = cells[3].split()
                return float(rd) * scale[ru] + float(wr) * scale[wu]
            except (ValueError, KeyError):
                return None
    return None


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
def time_device(disk, stream, steps, flush):
    """Device time of `steps` DTs.  Every step is enqueued ahead (as an
    application driving fargo_run_async does): an L2 flush, then one DT graph
    between two events; only the graphs' intervals are summed, and the host
    synchronises once after the last step."""
    import torch
    sc0 = disk.scalars()
    s0, p0 = sc0.substeps, sc0.padded_substeps
    events = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        disk.run_async(1)
        e1.record(stream)
        events.append((e0, e1))
    stream.synchronize()
    times = [e0.elapsed_time(e1) for e0, e1 in events]
    disk.sync()
    sc1 = disk.scalars()
    return sum(times), sc1.substeps - s0, sc1.padded_substeps - p0


def time_e2e(disk, stream, steps, params):
    """Through the C-ABI with host buffers: pinned FP64 host arrays are copied in,
    one DT runs, the fields are copied out, every step."""
    import ctypes

    import numpy as np
    import torch
    shape = (params.nrad + 1, params.nsec)
    names = ["dens", "vrad", "vtheta"] + (["energy"] if params.adiabatic else [])
    host = {n: torch.from_numpy(disk.field(n)).pin_memory() for n in names}
    ptr = {n: ctypes.cast(host[n].data_ptr(), ctypes.POINTER(ctypes.c_double)) for n in names}
    lib, h = disk.lib, disk.h
    nbytes = int(np.prod(shape)) * 8
    disk.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    s0 = disk.scalars().substeps
    e0.record(stream)
    t0 = time.perf_counter()
    for _ in range(steps):
        rc = lib.fargo_set_fields(h, ptr["dens"], ptr["vrad"], ptr["vtheta"], ptr.get("energy"))
        assert rc == 0
        n = ctypes.c_int(0)
        rc = lib.fargo_step_DT(h, ctypes.byref(n))
        assert rc == 0, lib.fargo_last_error(h)
        rc = lib.fargo_get_fields(h, ptr["dens"], ptr["vrad"], ptr["vtheta"], ptr.get("energy"), None)
        assert rc == 0
    e1.record(stream)
    e1.synchronize()
    wall = time.perf_counter() - t0
    nsub = disk.scalars().substeps - s0
    return wall, nsub, len(names) * nbytes, len(names) * nbytes


def batch_ensemble(ndt=2, n=64):
    """The batched ensemble (64 seeded disks, Nrad in {128..512}, Nsec = 3 Nrad):
    FP32-bulk disks advanced side by side (fargo_batch) against the same disks in
    plain FP64 one after another, after one warm-up DT each; the FP32 density
    error against FP64 after the same DTs.  The ensemble's state (~1.4 GB FP32)
    is larger than L2; the plain runs flush L2 before each disk."""
    import numpy as np
    import torch
    import cudaprotoplanetarydisks_gb300 as fg
    disks = fg.c4_disks(n)
    cells = [p.nrad * p.nsec for p, _ in disks]

    def batched(variant):
        b = fg.Batch(disks, fg.FARGO_FP32_BULK, variant=variant)
        b.run_async(1)
        b.sync()
        s0 = [d.scalars().substeps for d in b.disks]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b.run_async(ndt)
        b.sync()
        t = time.perf_counter() - t0
        cu = sum((d.scalars().substeps - s0[k]) * cells[k] for k, d in enumerate(b.disks))
        dens = [d.field("dens")[:-1] for d in b.disks]
        launches = sum(d.scalars().launches_per_substep * (d.scalars().substeps - s0[k] + d.scalars().padded_substeps)
                       for k, d in enumerate(b.disks))
        b.close()
        return t, cu, dens, launches

    t32, cu32, dens32, launches32 = batched(None)
    # the schedule autotuner (fargo_batch_autotune), then the tuned variant timed as above
    t_tune = time.perf_counter()
    variant, r_best, r_default = fg.autotune(disks, fg.FARGO_FP32_BULK, ndt=1)
    t_tune = time.perf_counter() - t_tune
    tt, cut, dens_t, _ = batched(variant)
    assert all(np.array_equal(x, y) for x, y in zip(dens32, dens_t))  # variants change speed only
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    t64, cu64, err = 0.0, 0, []
    for k, (p, pl) in enumerate(disks):
        d = fg.Disk(p, pl, fg.FARGO_FP64)
        d.run(1)
        s = d.scalars().substeps
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d.run(ndt)
        t64 += time.perf_counter() - t0
        cu64 += (d.scalars().substeps - s) * cells[k]
        ref = d.field("dens")[:-1]
        err.append(float(np.linalg.norm(dens32[k] - ref) / np.linalg.norm(ref)))
        d.close()
    v32, v64 = cu32 / t32, cu64 / t64
    return {"workload": f"{n} seeded disks, Nrad in {{128,192,256,384,512}}, Nsec = 3 Nrad, isothermal, "
                        "alpha, one planet each (configs c4_disks)",
            "cells": sum(cells), "dts_per_disk": ndt,
            "fp32_batched": {"value": v32, "unit": METRIC, "seconds": t32, "gpu_launches_approx": launches32},
            "fp32_batched_autotuned": {"value": cut / tt, "unit": METRIC, "seconds": tt, "variant": variant.as_dict(),
                                       "search": {"seconds": t_tune, "rate_default": r_default, "rate_kept": r_best}},
            "fp64_plain_sequential": {"value": v64, "unit": METRIC, "seconds": t64},
            "ratio_fp32_batched_to_fp64_plain": v32 / v64,
            "fp32_dens_rel_l2_vs_fp64_max": max(err), "fp32_dens_rel_l2_vs_fp64_median": float(np.median(err)),
            "timing": "host wall clock around run + sync (many streams: one per disk)"}


def learned_c5():
    """The learned coarse-grid correction: 256 x 768 disks of the ensemble
    distribution with a 4x finer plain run as teacher.  Training pairs come from
    the plain solver; on held-out disks: the one-DT loss with and without the
    network, a 10-DT rollout from the restricted teacher state (density relative
    L2 against the restricted teacher after 1 and 10 DTs, plain and learned), the
    wall time per DT of teacher, plain and learned runs; and the MLP kernels'
    throughput on one 256 x 768 disk's rows (CUDA events, 50 launches)."""
    from cudaprotoplanetarydisks_gb300 import learned as L
    r = L.experiment()
    kernels = L.kernel_timing()
    fe = r["field_err_rel_per_dt"]
    return {
        "workload": r["workload"],
        "train": r["train"],
        "held_out_one_dt_loss": r["held_out_one_dt_loss"],
        "rollout_dens_rel_l2": {"after_1_dt": {"plain": fe["plain"][0], "learned": fe["learned"][0]},
                                f"after_{r['rollout_dts']}_dts": {"plain": fe["plain"][-1],
                                                                  "learned": fe["learned"][-1]}},
        "profile_rel_l2_after_rollout": r["profile_err_rel"],
        "s_per_dt": r["s_per_dt"],
        "corrections": r["corrections"],
        "mlp_kernels": kernels,
    }


def oracle_sample(params, planets, ndt, threads):
    from oracle.oracle import OracleDisk
    OracleDisk.set_threads(threads)
    o = OracleDisk(params, planets)
    t0 = time.perf_counter()
    n = 0
    for _ in range(ndt):
        n += o.step_DT()
    dt = time.perf_counter() - t0
    return o, n, dt


def run_own(args, world, rank, local):
    import numpy as np
    import torch

    import cudaprotoplanetarydisks_gb300 as fg
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    params, planets, wname = workload(args.config)
    cells = params.nrad * params.nsec
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()

    results = {}
    for prec, key in ((fg.FARGO_FP32_BULK, "fp32"), (fg.FARGO_FP64, "fp64")):
        disk = fg.Disk(params, planets, prec, stream=stream.cuda_stream)
        for _ in range(args.warmup):
            disk.run(1)
        sampler = ClockSampler(local) if key == "fp32" else None
        barrier()
        if sampler:
            sampler.start()
        ms, nsub, npad = time_device(disk, stream, args.steps, flush)
        barrier()
        clocks = sampler.stop() if sampler else None
        ms_max, nsub_all = reduce_over_ranks(ms, nsub)
        r = {"ms_total": ms_max, "substeps": nsub_all, "value": job_value(nsub_all, cells, ms_max),
             "ms_per_step": ms_max / args.steps, "substeps_per_step": nsub / args.steps}
        sc = disk.scalars()
        # padded substeps (dt = 0, filling a loop body of two) launch their kernels too
        r["launches"] = int(args.steps * sc.launches_per_dt + (nsub + npad) * sc.launches_per_substep)
        r["padded_substeps"] = npad
        if key == "fp32":
            r["clocks"] = clocks
            wall, n_e2e, bi, bo = time_e2e(disk, stream, args.steps, params)
            r["e2e"] = {"value": n_e2e * cells * world / wall, "unit": METRIC,
                        "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo, "ms_per_step": wall * 1e3 / args.steps}
        # per-kernel device time (launch by launch, after the timed region)
        ms_k = (ctypes.c_double * 96)()
        nk = ctypes.c_int(0)
        rc = disk.lib.fargo_time_substep_kernels(disk.h, 5, ms_k, 96, ctypes.byref(nk))
        kern = []
        if rc == 0:
            for k in range(nk.value):
                nm = disk.lib.fargo_substep_kernel_name(disk.h, k).decode()
                kern.append((nm, ms_k[k]))
        r["kernels"] = kern
        disk.close()
        results[key] = r
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    hbm_peak, peak_kind = measured_peaks()
    f32 = results["fp32"]
    # dominant kernel of the headline mode, with its algorithmic bytes
    agg = {}
    for nm, t in f32["kernels"]:
        a = agg.setdefault(nm, [0.0, 0])
        a[0] += t
        a[1] += 1
    # k_planets runs on a second stream beside the hydro kernels (outside a
    # corotating frame), off the substep's critical path
    crit = {k: v for k, v in agg.items() if not (k == "k_planets" and not params.corotating)}
    dom = max(crit.items(), key=lambda kv: kv[1][0]) if crit else ("none", [1.0, 1])
    dom_name, (dom_ms, dom_n) = dom
    dom_avg_ms = dom_ms / dom_n
    alg = kernel_bytes(dom_name, params, 4)
    achieved = alg / (dom_avg_ms * 1e-3) / 1e9
    step_alg = 24 + (128 if params.self_gravity else 0) + (8 if params.adiabatic else 0)
    line = {
        "metric": METRIC, "value": f32["value"], "unit": "cell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": f32["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32",
        "precision_detail": "f32 fields and self-gravity FFT; f64 CFL decision, planets, ring means, FARGO "
                            "split; compensated f32 (float-float) force and ring sums",
        "data": "synthetic (seeded 1e-3 uniform noise on Sigma, reference .par/.cfg interface)",
        "config": config_obj(params, wname, args.config,
                             {"precision": "FP32_BULK", "parallelism": f"replicas x{world}",
                              "substeps_per_step": f32["substeps_per_step"]}),
        "e2e": f32["e2e"],
        "gpu_launches": f32["launches"],
        "clocks": f32["clocks"],
        "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": hbm_peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm_peak,
                     "alg_bytes_per_launch": alg, "avg_launch_ms": dom_avg_ms,
                     "traffic": ncu_traffic(dom_name, args.config),
                     "traffic_source": f"profiles/kernels_{args.config}_fp32.md (ncu, one cold-cache launch)"},
        "step_roofline": {"alg_bytes_per_cell_update": step_alg,
                          "achieved_GBs": f32["value"] * step_alg / 1e9,
                          "frac": f32["value"] * step_alg / 1e9 / hbm_peak},
        "kernels_ms": {nm: round(t / n, 5) for nm, (t, n) in agg.items()},
        "fp64": {"value": results["fp64"]["value"], "ms_per_step": results["fp64"]["ms_per_step"],
                 "gpu_launches": results["fp64"]["launches"],
                 "kernels_ms": {nm: round(t, 5) for nm, t in results["fp64"]["kernels"]}},
    }
    # CPU baseline (oracle, all host cores) on a bounded sample, and the FP32 error
    # against the FP64 oracle after the same DTs
    if not args.no_cpu_baseline:
        import numpy as np
        ndt = 2
        cores = os.cpu_count() or 1
        o, n_cpu, t_cpu = oracle_sample(params, planets, ndt, cores)
        line["cpu_baseline"] = {"value": n_cpu * cells / t_cpu, "unit": METRIC, "cores": cores, "kind": "port",
                                "sample": f"{ndt} DTs ({n_cpu} substeps) of the same disk from its initial state"}
        disk = fg.Disk(params, planets, fg.FARGO_FP32_BULK, stream=stream.cuda_stream)
        for _ in range(ndt):
            disk.step_DT()
        err = {}
        for nm in ("dens", "vrad", "vtheta"):
            a, b = disk.field(nm)[:-1], o.field(nm)[:-1]
            err[nm] = {"rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                       "rel_linf": float(np.abs(a - b).max() / np.abs(b).max())}
        line["fp32_error_vs_fp64_oracle"] = {"after": f"{ndt} DTs", "fields": err}
        disk.close()
        o.close()
    if not args.no_batch and world == 1:
        line["batch_c4"] = batch_ensemble()
    if not args.no_learned and world == 1:
        line["learned_c5"] = learned_c5()
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_reference(args, world, rank):
    if rank != 0:
        return
    params, planets, wname = workload(args.config)
    cells = params.nrad * params.nsec
    cores = os.cpu_count() or 1
    from oracle.oracle import OracleDisk
    OracleDisk.set_threads(cores)
    o = OracleDisk(params, planets)
    for _ in range(args.warmup):
        o.step_DT()
    # a bounded sample: the first timed DT sets how many fit in REF_BUDGET_S
    t0 = time.perf_counter()
    n = o.step_DT()
    steps = 1
    cap = max(1, min(args.steps, int(REF_BUDGET_S / max(time.perf_counter() - t0, 1e-9))))
    while steps < cap:
        n += o.step_DT()
        steps += 1
    dt = time.perf_counter() - t0
    value = n * cells / dt
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "impl": "reference", "dtype": "f64",
        "data": "synthetic (seeded 1e-3 uniform noise on Sigma, reference .par/.cfg interface)",
        "config": config_obj(params, wname, args.config, {"precision": "FP64", "parallelism": "host cores"}),
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "port",
                         "sample": f"{steps} of the {args.steps} requested DTs ({n} substeps, about "
                                   f"{REF_BUDGET_S:.0f} s at most) after {args.warmup} warm-up DTs"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference runs every substep as a CUDA kernel and has no CPU path; "
                "this arm times its CPU restatement (the oracle) with OpenMP over rings",
    }
    print(json.dumps(line), flush=True)


def run_profile(args):
    import cudaprotoplanetarydisks_gb300 as fg
    params, planets, _ = workload(args.config)
    prec = fg.FARGO_FP32_BULK if args.profile == "fp32" else fg.FARGO_FP64
    disk = fg.Disk(params, planets, prec)
    for _ in range(args.warmup):
        disk.run(1)
    ms = (ctypes.c_double * 96)()
    nk = ctypes.c_int(0)
    rc = disk.lib.fargo_time_substep_kernels(disk.h, args.steps, ms, 96, ctypes.byref(nk))
    assert rc == 0, disk.lib.fargo_last_error(disk.h)
    for k in range(nk.value):
        print(f"{disk.lib.fargo_substep_kernel_name(disk.h, k).decode():28s} {ms[k] * 1e3:9.2f} us")
    disk.close()


def main():
    args = parse()
    world, rank, local = dist_env()
    if args.profile:
        run_profile(args)
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_own(args, world, rank, local)


if __name__ == "__main__":
    main()
