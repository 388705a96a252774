#!/usr/bin/env python
"""Benchmark of the FARGO-ADSG hydro step on GB300.

Workload (default, --config c3): the adiabatic disk with cooling, 1024 x 3072
log grid on [0.3, 3.0], gamma = 1.4, cooling time 10 r^(2+2f), alpha = 1e-3,
Sigma ~ r^-0.5, one planet q = 1e-3 on a fixed circular orbit at r = 1, seeded
1e-4 noise on Sigma and energy (cudaprotoplanetarydisks_gb300/configs/
c3_adiabatic.par), the largest single-disk configuration of the benchmark set.
A step is one DT (AlgoGas: CFL-subcycled hydro substeps); the metric counts cell
updates, Nrad * Nsec per hydro substep.

Own arm, headline: the FP64 mode (the reference's arithmetic).  The state stays
in HBM (about 0.5 GB, above the 129 MB L2); each timed step is one graph launch of
a DT (CFL loop on the device), timed with CUDA events on the launching stream,
with an L2 flush (a 256 MiB write) before every timed step.  e2e: the same metric
through the C-ABI with host buffers (pinned FP64 arrays copied in and out every
step).  Beside it: the FP32-bulk mode (own value, e2e and field errors against
the FP64 mode after the same DTs), the self-gravitating 256 x 768 disk in both
modes, the batched ensemble and the learned correction.  The roofline of the
FP64 mode is its FP64 pipe (measured peak: fargo_fp64_pipe_peak).

CPU baselines: the reference's own sources compiled for the CPU
(oracle/_ref/fargo_ref_cpu, blocks of each launch on the host cores) on a bounded
sample of the same disk -- the DT shortened to about one hydro substep, so that
each AlgoGas call is a sample of the workload's substeps -- on all host cores and
on one; and the oracle (the C++ restatement) on all host cores.

--impl reference: the reference's own code on the host cores (the CPU build
above), on the same workload and metric, never loading this package's library.

--gpus N (torchrun, one rank per GPU): replicas only -- every rank advances its
own disk; value = all ranks' cell updates / the slowest rank's time.
"""
import argparse
import ctypes
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-updates/s"
L2_FLUSH_BYTES = 256 << 20
CONFIG_DIR = os.path.join(ROOT, "cudaprotoplanetarydisks_gb300", "configs")
CONFIG_FILES = {"c1": "c1_isothermal.par", "c2": "c2_selfgravity.par", "c3": "c3_adiabatic.par",
                "wide": "wide_template4.par"}
WORKLOADS = {"c1": "isothermal disk 128x384, 1 planet (fixed orbit)",
             "c2": "self-gravitating disk 256x768, alpha viscosity, migrating planet",
             "c3": "adiabatic disk with cooling 1024x3072, alpha viscosity, 1 planet (fixed orbit)",
             "wide": "adiabatic disk 2048x4096, non-reflecting inner boundary, guiding-center frame, "
                     "Jupiter-mass planet"}
# the CPU samples' DT is the workload's DT over this divisor: about one hydro
# substep per AlgoGas call (twice the substeps per DT measured on the workload,
# as the first substeps of a run take a smaller CFL step)
SAMPLE_DT_DIVISOR = {"c1": 30, "c2": 54, "c3": 220, "wide": 200}
REF_EXE = os.path.join(ROOT, "oracle", "_ref", "fargo_ref_cpu")
REF_CUDA_EXE = os.path.join(ROOT, "oracle", "_ref", "fargoGPU_sm103a")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c3")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the 256x768 self-gravitating disk extra")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="skip the reference's own CUDA build on the isothermal 128x384 disk")
    ap.add_argument("--no-drift", action="store_true", help="skip the 100-orbit FP32-bulk drift measurement")
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
    return params, planets, WORKLOADS.get(cfg, cfg)


def config_obj(params, name, cfg, extra=None):
    c = {"workload": name, "config_file": f"configs/{CONFIG_FILES.get(cfg, cfg)}", "nrad": params.nrad,
         "nsec": params.nsec, "cells": params.nrad * params.nsec, "self_gravity": bool(params.self_gravity),
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
        "k_energy": 4 + 3,  # vrad, vtheta, dens, energyint in; divv, qplus, energy out
        "k_transport_radial": (3 + ad) + (5 + ad),
        "k_transport_radial_tma": (3 + ad) + (5 + ad),
        "k_transport_radial_col": (3 + ad) + (5 + ad),
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


def _profile_rows(cfg, mode):
    """Rows (cells split on '|') of the committed ncu summary
    profiles/kernels_<cfg>_<mode>.md, keyed by kernel name without template
    arguments."""
    path = os.path.join(ROOT, "profiles", f"kernels_{cfg}_{mode}.md")
    rows = {}
    if not os.path.exists(path):
        return rows
    for line in open(path):
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cells) >= 4:
            rows.setdefault(cells[0].split("<")[0], cells)
    return rows


def ncu_traffic(kernel, cfg, mode="fp32"):
    """DRAM bytes (read + write) of one launch of `kernel` from the committed ncu
    summary profiles/kernels_<cfg>_<mode>.md (one cold-cache capture), or None."""
    rows = _profile_rows(cfg, mode)
    # the substep timer names both azimuthal forms k_transport_azimuthal; ncu names
    # the register form k_transport_azimuthal4
    cells = rows.get(kernel) or rows.get(kernel + "4")
    if cells is None:
        return None
    try:  # columns: kernel, launches, avg us, read MB, write MB, ...
        return (float(cells[3]) + float(cells[4])) * 1e6
    except (ValueError, IndexError):
        pass
    scale = {"B": 1.0, "KB": 1e3, "MB": 1e6, "GB": 1e9}
    try:
        rd, ru = cells[2].split()
        wr, wu = cells[3].split()
        return float(rd) * scale[ru] + float(wr) * scale[wu]
    except (ValueError, KeyError):
        return None


def ncu_fp64_instructions(kernel, cfg):
    """FP64-pipe thread instructions of one launch of `kernel` (warp instructions
    x 32) from the committed ncu summary profiles/kernels_<cfg>_fp64.md, or None."""
    cells = _profile_rows(cfg, "fp64").get(kernel)
    try:
        return float(cells[6]) * 32.0
    except (TypeError, ValueError, IndexError):
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


def kernel_times(disk, reps=3):
    """Per-kernel device time of one substep, launch by launch (CUDA events between
    kernels), after the timed region: [(name, ms)]."""
    ms_k = (ctypes.c_double * 96)()
    nk = ctypes.c_int(0)
    rc = disk.lib.fargo_time_substep_kernels(disk.h, reps, ms_k, 96, ctypes.byref(nk))
    if rc != 0:
        return []
    return [(disk.lib.fargo_substep_kernel_name(disk.h, k).decode(), ms_k[k]) for k in range(nk.value)]


def dominant(kern, params):
    """The kernel with the largest device time per substep on the critical path
    (k_planets runs on a second stream beside the hydro kernels outside a
    corotating frame): (name, total ms per substep, launches per substep)."""
    agg = {}
    for nm, t in kern:
        a = agg.setdefault(nm, [0.0, 0])
        a[0] += t
        a[1] += 1
    crit = {k: v for k, v in agg.items() if not (k == "k_planets" and not params.corotating)}
    if not crit:
        return "none", 1.0, 1, agg
    nm, (ms, n) = max(crit.items(), key=lambda kv: kv[1][0])
    return nm, ms, n, agg


def step_alg_bytes(params, esize):
    """Algorithmic bytes per cell update of the whole step: every state field read
    and written once per substep (+ the self-gravity FFT round trips)."""
    nf = 3 + (1 if params.adiabatic else 0)
    return 2 * nf * esize + (128 if params.self_gravity else 0)


def measure_mode(fg, params, planets, prec, stream, flush, steps, warmup, clocks_gpu=None, e2e=True):
    """One precision mode on one disk: device-resident value, e2e through the
    C-ABI, launches in the timed region and per-kernel times."""
    disk = fg.Disk(params, planets, prec, stream=stream.cuda_stream)
    for _ in range(warmup):
        disk.run(1)
    sampler = ClockSampler(clocks_gpu) if clocks_gpu is not None else None
    import torch
    torch.cuda.synchronize()
    if sampler:
        sampler.start()
    ms, nsub, npad = time_device(disk, stream, steps, flush)
    torch.cuda.synchronize()
    r = {"ms": ms, "substeps": nsub, "padded_substeps": npad}
    if sampler:
        r["clocks"] = sampler.stop()
    sc = disk.scalars()
    # padded substeps (dt = 0, filling a loop body of two) launch their kernels too
    r["launches"] = int(steps * sc.launches_per_dt + (nsub + npad) * sc.launches_per_substep)
    if e2e:
        wall, n_e2e, bi, bo = time_e2e(disk, stream, steps, params)
        r["e2e"] = (wall, n_e2e, bi, bo)
    r["kernels"] = kernel_times(disk)
    disk.close()
    return r


def fp32_errors(fg, params, planets, stream, ndt=2):
    """Per-field relative L2 / Linf error of the FP32-bulk mode against the FP64
    mode of the same code after the same DTs from the same initial state (the FP64
    mode matches the oracle within 1e-9: tests/test_gpu_parity.py)."""
    import numpy as np
    d32 = fg.Disk(params, planets, fg.FARGO_FP32_BULK, stream=stream.cuda_stream)
    d64 = fg.Disk(params, planets, fg.FARGO_FP64, stream=stream.cuda_stream)
    d32.run(ndt)
    d64.run(ndt)
    names = ["dens", "vrad", "vtheta"] + (["energy"] if params.adiabatic else [])
    err = {}
    for nm in names:
        a, b = d32.field(nm)[:-1], d64.field(nm)[:-1]
        err[nm] = {"rel_l2": float(np.linalg.norm(a - b) / np.linalg.norm(b)),
                   "rel_linf": float(np.abs(a - b).max() / np.abs(b).max())}
    d32.close()
    d64.close()
    return {"after": f"{ndt} DTs", "against": "FP64 mode of this code", "fields": err}


# ---------------------------------------------------------------------------
# the reference's own sources on the CPU (oracle/_ref/fargo_ref_cpu)
def _par_values(text):
    vals = {}
    for line in text.splitlines():
        parts = line.split()
        if len(parts) >= 2 and not parts[0].startswith("#"):
            vals[parts[0].upper()] = parts[1]
    return vals


def run_reference_exe(exe, cfg, ndt, env_extra=None, dt_divisor=1.0, ninterm=1000000000, outdir=None, overrides=None,
                      planet_mass=None):
    """Runs a build of the reference's main() (oracle/_ref: its CPU build or its own
    CUDA build) on the workload's .par for ndt DTs (Ntot = ndt - 1: the reference
    runs Ntot + 1), the DT divided by dt_divisor, dumps every `ninterm` DTs into
    outdir (a temporary directory when None), the seeded noise of the .par's
    SigmaNoise / EnergyNoise / NoiseSeed keys through the build's link-time
    wrappers; overrides replaces .par keys (e.g. {"NRAD": 128, "NSEC": 384}) and
    planet_mass the mass column of the planet file.
    Returns ([(substeps, AlgoGas seconds) per DT], cells) from the binary's
    REFSTEP lines.  Reads no product code."""
    if not os.path.exists(exe):
        raise RuntimeError(f"{exe} is missing (built by build(): oracle/ref_emul, oracle/ref_cuda)")
    src = os.path.join(CONFIG_DIR, CONFIG_FILES[cfg])
    text = open(src).read()
    over = {k.upper(): v for k, v in (overrides or {}).items()}
    if over:
        lines, seen = [], set()
        for line in text.splitlines():
            k = line.split()[0].upper() if line.split() else ""
            lines.append(f"{k} {over[k]}" if k in over else line)
            seen.add(k)
        lines += [f"{k} {v}" for k, v in over.items() if k not in seen]
        text = "\n".join(lines) + "\n"
    vals = _par_values(text)
    with tempfile.TemporaryDirectory() as d:
        out = outdir or os.path.join(d, "out")
        os.makedirs(out, exist_ok=True)
        keep = []
        for line in text.splitlines():
            k = line.split()[0].upper() if line.split() else ""
            if k in ("NTOT", "NINTERM", "DT", "OUTPUTDIR", "PLANETCONFIG"):
                continue
            keep.append(line)
        keep += [f"Ntot {ndt - 1}", f"Ninterm {int(ninterm)}",
                 f"DT {float(vals.get('DT', '0.314159265359')) / dt_divisor!r}", f"OutputDir {out}/"]
        if "PLANETCONFIG" in vals:
            # the reference keeps the planet file's path in a fixed-size buffer
            # (src/Main.cu:248-249): a short copy beside the run
            cfg_path = os.path.join(d, "planet.cfg")
            with open(os.path.join(CONFIG_DIR, vals["PLANETCONFIG"])) as f_in, open(cfg_path, "w") as f_out:
                for line in f_in.read().splitlines():
                    tok = line.split()
                    if planet_mass is not None and tok and not tok[0].startswith("#") and len(tok) >= 3:
                        tok[2] = repr(float(planet_mass))
                        line = "  ".join(tok)
                    f_out.write(line + "\n")
            keep.append(f"PlanetConfig {cfg_path}")
        par = os.path.join(d, "run.par")
        open(par, "w").write("\n".join(keep) + "\n")
        env = dict(os.environ)
        env.update(env_extra or {})
        for key, var in (("SIGMANOISE", "FARGO_REF_SIGMA_NOISE"), ("ENERGYNOISE", "FARGO_REF_ENERGY_NOISE"),
                         ("NOISESEED", "FARGO_REF_NOISE_SEED")):
            if key in vals:
                env[var] = vals[key]
        r = subprocess.run([exe, par], input="0\n", capture_output=True, text=True, env=env, cwd=d,
                           timeout=3600)
        if r.returncode != 0:
            raise RuntimeError(f"{os.path.basename(exe)} failed ({r.returncode}): {(r.stdout + r.stderr)[-600:]}")
        steps = [m.groups() for m in re.finditer(r"REFSTEP (\d+) (\d+) ([0-9.eE+-]+)", r.stderr)]
    cells = int(vals["NRAD"]) * int(vals["NSEC"])
    return [(int(s), float(t)) for _, s, t in steps], cells


def reference_cpu_sample(cfg, ndt, threads, sample_divisor=None):
    """The reference's CPU build on a bounded sample of the workload: the DT
    shortened to about one hydro substep, on `threads` host threads (blocks of
    each launch in parallel).  Returns ([(substeps, seconds) per DT], cells, divisor)."""
    divisor = sample_divisor or SAMPLE_DT_DIVISOR.get(cfg, 100)
    steps, cells = run_reference_exe(REF_EXE, cfg, ndt, {"FARGO_REF_THREADS": str(threads),
                                                         "OMP_NUM_THREADS": str(threads)}, dt_divisor=divisor)
    return steps, cells, divisor


def reference_cuda(fg, stream, flush):
    """The reference's own CUDA build (oracle/_ref/fargoGPU_sm103a, sm_103a, two
    source-compat fixes) on the isothermal 128 x 384 disk -- the one configuration
    whose kernels were read for out-of-bounds access -- for 15 DTs (about 220 hydro
    substeps, the first DT untimed), timed by the AlgoGas wrapper; beside it, this
    code's FP64 mode on the same disk and DTs, device-resident and through the C-ABI."""
    if not os.path.exists(REF_CUDA_EXE):
        err = REF_CUDA_EXE + ".build_error"
        return {"unavailable": open(err).read()[-300:] if os.path.exists(err) else f"{REF_CUDA_EXE} not built"}
    steps, cells = run_reference_exe(REF_CUDA_EXE, "c1", 15)
    n, t = sum(s for s, _ in steps[1:]), sum(x for _, x in steps[1:])
    p1, pl1, _ = workload("c1")
    r = measure_mode(fg, p1, pl1, fg.FARGO_FP64, stream, flush, 14, 1)
    w, ne, _, _ = r["e2e"]
    own = r["substeps"] * cells / (r["ms"] * 1e-3)
    out = {"workload": WORKLOADS["c1"], "config_file": "configs/" + CONFIG_FILES["c1"],
           "build": "the reference's src/*.cu with nvcc 13 for sm_103a (Makefile flags; __shfl_down_sync and "
                    "::array compat fixes), seeded noise and AlgoGas timing through link-time wrappers",
           "value": n * cells / t, "unit": METRIC, "dtype": "f64", "substeps": n, "seconds": t,
           "timing": "host clock around each AlgoGas call (the reference synchronises the device after every "
                     "launch), DTs 2..15",
           "gb300_fp64_same_disk": {"value": own, "e2e": ne * cells / w, "unit": METRIC,
                                    "ms_per_dt": r["ms"] / 14}}
    # the headline disk (1024 x 3072 adiabatic with cooling, WALL boundaries, no
    # self-gravity: its kernels read for out-of-bounds access too), 3 DTs, the
    # first untimed; this code's FP64 on the same disk is the headline value
    steps3, cells3 = run_reference_exe(REF_CUDA_EXE, "c3", 3)
    n3, t3 = sum(s for s, _ in steps3[1:]), sum(x for _, x in steps3[1:])
    out["c3"] = {"workload": WORKLOADS["c3"], "config_file": "configs/" + CONFIG_FILES["c3"],
                 "value": n3 * cells3 / t3, "unit": METRIC, "dtype": "f64", "substeps": n3, "seconds": t3,
                 "timing": "host clock around each AlgoGas call, DTs 2..3"}
    out["c4_sequential"] = reference_cuda_c4()
    return out


def c4_overrides(d):
    """.par keys of an ensemble disk (config.c4_draws) over the isothermal c1 file."""
    return {"NRAD": d["nrad"], "NSEC": d["nsec"], "VISCOSITY": 0.0, "ALPHAVISCOSITY": repr(d["alpha"]),
            "ASPECTRATIO": repr(d["h"]), "SIGMASLOPE": repr(d["slope"]), "SIGMA0": 6.3662e-4,
            "SIGMANOISE": 1e-4, "NOISESEED": d["noise_seed"]}


def reference_cuda_c4(n=64, ndt=2):
    """The ensemble's baseline: the 64 disks of the batched workload as 64
    sequential runs of the reference's own CUDA build (isothermal, alpha viscosity,
    WALL boundaries, no self-gravity: the kernels read for out-of-bounds access),
    one process each, ndt DTs with the first untimed.  The disks' draws come from
    config.c4_draws; .par keys per disk, the planet file's mass per disk."""
    from cudaprotoplanetarydisks_gb300.config import c4_draws
    tot_n = tot_t = 0.0
    subs = 0
    for d in c4_draws(n):
        steps, cells = run_reference_exe(REF_CUDA_EXE, "c1", ndt, overrides=c4_overrides(d), planet_mass=d["q"])
        ns = sum(s for s, _ in steps[1:])
        subs += ns
        tot_n += ns * cells
        tot_t += sum(x for _, x in steps[1:])
    return {"workload": f"the {n} seeded disks of batch_c4 (Nrad 128-512, Nsec = 3 Nrad, isothermal, alpha, one "
                        "planet each), one reference process per disk, one after another",
            "value": tot_n / tot_t, "unit": METRIC, "dtype": "f64", "substeps": subs, "seconds": tot_t,
            "timing": f"host clock around each AlgoGas call, DTs 2..{ndt} of every disk (process start-up and "
                      "set-up not counted)"}


def cpu_baselines(cfg, params, planets):
    """cpu_baseline (the reference's own code, all host cores) plus the one-core
    figure and the oracle (C++ restatement) on all host cores, each on a bounded
    sample of the workload."""
    cores = os.cpu_count() or 1
    out = {}
    steps, cells, div = reference_cpu_sample(cfg, 3, cores)
    n, t = sum(s for s, _ in steps[1:]), sum(x for _, x in steps[1:])
    out["cpu_baseline"] = {"value": n * cells / t, "unit": METRIC, "cores": cores, "kind": "reference",
                           "sample": f"the reference's own sources compiled for the CPU (blocks of each launch "
                                     f"on {cores} host threads), DT shortened to DT/{div}: {n} hydro substeps "
                                     f"in 2 timed AlgoGas calls after 1 untimed"}
    steps1, _, _ = reference_cpu_sample(cfg, 1, 1)
    n1, t1 = sum(s for s, _ in steps1), sum(x for _, x in steps1)
    out["cpu_baseline_1core"] = {"value": n1 * cells / t1, "unit": METRIC, "cores": 1, "kind": "reference",
                                 "sample": f"the same build on one host thread: {n1} hydro substep(s) in one "
                                           f"AlgoGas call (DT/{div})"}
    from oracle.oracle import OracleDisk
    OracleDisk.set_threads(cores)
    p = type(params).from_buffer_copy(params)
    p.dt = params.dt / div
    o = OracleDisk(p, planets)
    t0 = time.perf_counter()
    no = o.step_DT() + o.step_DT()
    to = time.perf_counter() - t0
    o.close()
    out["cpu_baseline_port"] = {"value": no * cells / to, "unit": METRIC, "cores": cores, "kind": "port",
                                "sample": f"the oracle (C++ restatement, OpenMP over rings): {no} hydro substeps "
                                          f"(2 DTs of DT/{div})"}
    return out


# ---------------------------------------------------------------------------
def run_own(args, world, rank, local):
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

    # headline: FP64 (the reference's arithmetic), clocks sampled in its timed region
    barrier()
    r64 = measure_mode(fg, params, planets, fg.FARGO_FP64, stream, flush, args.steps, args.warmup,
                       clocks_gpu=local)
    barrier()
    ms_max, nsub_all = reduce_over_ranks(r64["ms"], r64["substeps"])
    r32 = measure_mode(fg, params, planets, fg.FARGO_FP32_BULK, stream, flush, args.steps, args.warmup)
    ms32_max, nsub32_all = reduce_over_ranks(r32["ms"], r32["substeps"])
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return
    hbm_peak, peak_kind = measured_peaks()
    value = job_value(nsub_all, cells, ms_max)
    wall, n_e2e, bi, bo = r64["e2e"]
    # roofline of the dominant FP64 kernel: HBM bytes, and its FP64 pipe (the bound)
    dname, dms, dn, agg64 = dominant(r64["kernels"], params)
    davg = dms / dn
    alg = kernel_bytes(dname, params, 8)
    achieved = alg / (davg * 1e-3) / 1e9
    dfma = ctypes.c_double(0.0)
    rc = fg._capi.load().fargo_fp64_pipe_peak(ctypes.byref(dfma))
    fp64_instr = ncu_fp64_instructions(dname, args.config)
    fp64_pipe = {"unit": "G FP64-pipe thread instructions/s", "peak": dfma.value / 1e9 if rc == 0 else None,
                 "peak_source": "fargo_fp64_pipe_peak (independent DFMA chains on every SM, measured in this run)",
                 "instructions_per_launch": fp64_instr,
                 "instructions_source": f"profiles/kernels_{args.config}_fp64.md (ncu sm__inst_executed_pipe_fp64 x 32)"}
    if fp64_instr and rc == 0:
        fp64_pipe["achieved"] = fp64_instr / (davg * 1e-3) / 1e9
        fp64_pipe["frac"] = fp64_pipe["achieved"] / fp64_pipe["peak"]
    sb64 = step_alg_bytes(params, 8)
    # FP32-bulk beside it
    d32, d32ms, d32n, agg32 = dominant(r32["kernels"], params)
    alg32 = kernel_bytes(d32, params, 4)
    ach32 = alg32 / (d32ms / d32n * 1e-3) / 1e9
    w32, n32e, bi32, bo32 = r32["e2e"]
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded uniform noise on Sigma and energy, reference .par/.cfg interface)",
        "config": config_obj(params, wname, args.config,
                             {"precision": "FP64", "parallelism": f"replicas x{world}",
                              "substeps_per_step": r64["substeps"] / args.steps}),
        "e2e": {"value": n_e2e * cells * world / wall, "unit": METRIC, "h2d_bytes_per_step": bi,
                "d2h_bytes_per_step": bo, "ms_per_step": wall * 1e3 / args.steps,
                "path": "fargo_set_fields + fargo_step_DT + fargo_get_fields (C-ABI, pinned FP64 host arrays)"},
        "gpu_launches": r64["launches"],
        "clocks": r64["clocks"],
        "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": hbm_peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm_peak,
                     "alg_bytes_per_launch": alg, "avg_launch_ms": davg,
                     "traffic": ncu_traffic(dname, args.config, "fp64"),
                     "traffic_source": f"profiles/kernels_{args.config}_fp64.md (ncu, one cold-cache launch)",
                     "fp64_pipe": fp64_pipe,
                     "note": "the FP64 kernels are bound by the FP64 pipe (77-88% busy in ncu), not by HBM; "
                             "fp64_pipe.frac is the roofline fraction that applies"},
        "step_roofline": {"alg_bytes_per_cell_update": sb64, "achieved_GBs": value * sb64 / 1e9,
                          "frac": value * sb64 / 1e9 / hbm_peak},
        "kernels_ms": {nm: round(t / n, 5) for nm, (t, n) in agg64.items()},
        "fp32_bulk": {
            "value": job_value(nsub32_all, cells, ms32_max), "unit": METRIC, "ms_per_step": ms32_max / args.steps,
            "dtype": "f32",
            "precision_detail": "f32 fields and arithmetic; f64 CFL decision, planets, ring means, FARGO split; "
                                "compensated f32 (float-float) force and ring sums",
            "e2e": {"value": n32e * cells * world / w32, "unit": METRIC, "h2d_bytes_per_step": bi32,
                    "d2h_bytes_per_step": bo32},
            "gpu_launches": r32["launches"],
            "roofline": {"bound": "hbm", "kernel": d32, "achieved": ach32, "peak": hbm_peak, "unit": "GB/s",
                         "frac": ach32 / hbm_peak, "alg_bytes_per_launch": alg32,
                         "avg_launch_ms": d32ms / d32n, "traffic": ncu_traffic(d32, args.config, "fp32")},
            "step_roofline": {"alg_bytes_per_cell_update": step_alg_bytes(params, 4),
                              "frac": job_value(nsub32_all, cells, ms32_max) * step_alg_bytes(params, 4)
                              / 1e9 / hbm_peak},
            "kernels_ms": {nm: round(t / n, 5) for nm, (t, n) in dominant(r32["kernels"], params)[3].items()},
            "error_vs_fp64": fp32_errors(fg, params, planets, stream),
        },
    }
    if not args.no_cpu_baseline:
        line.update(cpu_baselines(args.config, params, planets))
    if not args.no_reference_cuda and world == 1:
        try:
            line["reference_cuda"] = reference_cuda(fg, stream, flush)
        except Exception as e:  # reported, never fatal to the own arm
            line["reference_cuda"] = {"unavailable": str(e)[-300:]}
    if not args.no_extra and world == 1 and args.config != "c2":
        p2, pl2, n2 = workload("c2")
        e = {"workload": n2, "config_file": "configs/c2_selfgravity.par"}
        for prec, key in ((fg.FARGO_FP64, "fp64"), (fg.FARGO_FP32_BULK, "fp32_bulk")):
            r = measure_mode(fg, p2, pl2, prec, stream, flush, 50, args.warmup, e2e=(key == "fp64"))
            e[key] = {"value": r["substeps"] * p2.nrad * p2.nsec / (r["ms"] * 1e-3), "unit": METRIC,
                      "ms_per_step": r["ms"] / 50, "steps": 50}
            if "e2e" in r:
                w, ne, _, _ = r["e2e"]
                e[key]["e2e"] = ne * p2.nrad * p2.nsec / w
        e["fp32_error_vs_fp64"] = fp32_errors(fg, p2, pl2, stream)
        line["c2"] = e
    if not args.no_drift and world == 1:
        from cudaprotoplanetarydisks_gb300.drift import drift

        def drift_obj(cfg):
            dr = drift(cfg, 100, every=25, control=True)
            return {"workload": WORKLOADS[cfg], "dts": dr["dts"], "dens_rel_l2": dr["final_dens_rel_l2"],
                    "fields_after_100_orbits": {k: dr["by_orbit"][-1][k] for k in ("dens", "vrad", "vtheta")},
                    "dens_rel_l2_by_orbit": {r["orbits"]: r["dens"]["rel_l2"] for r in dr["by_orbit"]},
                    "control_dens_rel_l2_by_orbit": {r["orbits"]: r["control_dens"]["rel_l2"]
                                                     for r in dr["by_orbit"]},
                    "control32_dens_rel_l2_by_orbit": {r["orbits"]: r["control32_dens"]["rel_l2"]
                                                       for r in dr["by_orbit"]},
                    "seconds": dr["seconds_fp64"] + dr["seconds_fp32"]}
        d2 = drift_obj("c2")
        line["fp32_drift_100_orbits"] = {
            "against": "FP64 mode of this code from the same initial state",
            "control": "FP64 from the same state with the density perturbed by one unit in the last place: "
                       "how much the flow itself amplifies the smallest perturbation",
            "control32": "FP64 from the same state with the density perturbed by one FP32 rounding (2^-24): "
                         "how much the flow amplifies a single FP32-sized error",
            "target": 1e-5, "dens_rel_l2": d2["dens_rel_l2"], "c2": d2, "c1": drift_obj("c1")}
    if not args.no_batch and world == 1:
        line["batch_c4"] = batch_ensemble()
        line["batch_small"] = batch_small()
    if not args.no_learned and world == 1:
        line["learned_c5"] = learned_c5()
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_reference(args, world, rank):
    """The reference's own code on the host cores: its sources compiled for the CPU
    (oracle/_ref/fargo_ref_cpu), the blocks of each launch on every host thread,
    on the same workload and metric.  Each step is one AlgoGas call of a bounded
    sample (DT shortened to about one hydro substep); warm-up calls are untimed.
    Only rank 0 runs; this never loads the product library."""
    if rank != 0:
        return
    cfg = args.config
    cores = os.cpu_count() or 1
    steps, cells, div = reference_cpu_sample(cfg, args.warmup + args.steps, cores)
    timed = steps[args.warmup:]
    n, t = sum(s for s, _ in timed), sum(x for _, x in timed)
    value = n * cells / t
    vals = _par_values(open(os.path.join(CONFIG_DIR, CONFIG_FILES[cfg])).read())
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3 / max(1, len(timed)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "impl": "reference", "dtype": "f64",
        "data": "synthetic (seeded uniform noise on Sigma and energy, reference .par/.cfg interface)",
        "config": {"workload": WORKLOADS.get(cfg, cfg), "config_file": f"configs/{CONFIG_FILES.get(cfg, cfg)}",
                   "nrad": int(vals["NRAD"]), "nsec": int(vals["NSEC"]), "cells": cells, "precision": "FP64",
                   "step": f"one AlgoGas call with DT shortened to DT/{div} (about one hydro substep)",
                   "parallelism": "host cores"},
        "cpu_baseline": {"value": value, "unit": METRIC, "cores": cores, "kind": "reference",
                         "sample": f"{len(timed)} AlgoGas calls ({n} hydro substeps) after {args.warmup} untimed, "
                                   f"DT/{div}; the reference's sources compiled for the CPU, blocks of each "
                                   f"launch on {cores} host threads"},
        "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference runs every substep as a CUDA kernel and has no CPU path of its own; this arm runs "
                "its unmodified kernels and host code on the CPU through an emulation of the launch syntax "
                "(oracle/ref_emul), bitwise equal to the golden fixtures",
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def batch_small(ndt=4, n=256):
    """An ensemble of many small disks (256 seeded disks of the C4 distribution at
    Nrad in {32, 48, 64}), where a disk's kernels are a few CTAs each and the
    per-disk graphs are bound by launch and scheduling overheads: per-disk graphs
    against the fused form (one launch per kernel per ring width, and one for the
    whole ensemble), FP32-bulk, after one warm-up DT, host wall clock."""
    import numpy as np
    import torch
    import cudaprotoplanetarydisks_gb300 as fg
    disks = fg.c4_disks(n, seed=5, nrad_choices=(32, 48, 64))
    cells = [p.nrad * p.nsec for p, _ in disks]

    def run(fused):
        b = fg.Batch(disks, fg.FARGO_FP32_BULK)
        if fused:
            b.fuse(by_width=(fused == "width"))
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
        b.close()
        return cu / t, dens

    v0, d0 = run(None)
    vw, dw = run("width")
    v1, d1 = run("one")
    same = all(np.array_equal(x, y) for x, y in zip(d0, dw)) and all(np.array_equal(x, y) for x, y in zip(d0, d1))
    return {"workload": f"{n} seeded disks of the C4 distribution, Nrad in {{32,48,64}}, Nsec = 3 Nrad",
            "cells": sum(cells), "dts_per_disk": ndt, "unit": METRIC,
            "per_disk_graphs": v0, "fused_by_width": vw, "fused_one_lane": v1,
            "speedup_fused_by_width": vw / v0, "speedup_fused_one_lane": v1 / v0,
            "bitwise_equal": same, "timing": "host wall clock around run + sync"}


def batch_ensemble(ndt=4, n=64):
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

    def batched(variant, fused=None, precision=None):
        b = fg.Batch(disks, fg.FARGO_FP32_BULK if precision is None else precision, variant=variant)
        if fused:
            b.fuse(by_width=(fused == "width"))
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
        if fused:
            per_sub, per_dt = b.fused_launches()
            nsub_max = max(d.scalars().substeps - s0[k] for k, d in enumerate(b.disks))
            launches = ndt * per_dt + nsub_max * per_sub  # at least: the loop runs to the slowest disk
            if fused == "width":
                # per-group device times of one substep (lanes one after another)
                groups = {}
                for name, ms in b.fused_kernel_times(reps=3):
                    groups[name] = groups.get(name, 0.0) + ms
                launches = (launches, {k: round(v, 4) for k, v in sorted(groups.items(), key=lambda kv: -kv[1])})
        else:
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
    # the fused forms: each substep kernel launched once per ring width (lanes side
    # by side), and once for the whole ensemble
    tf, cuf, dens_f, (launches_f, groups_ms) = batched(None, fused="width")
    fused_diff = max(float(np.abs(x - y).max() / np.abs(y).max()) for x, y in zip(dens_f, dens32))
    tf1, cuf1, dens_f1, launches_f1 = batched(None, fused="one")
    # FP64 at the same batching (per-disk graphs side by side)
    t64b, cu64b, _, _ = batched(None, precision=fg.FARGO_FP64)
    fused_diff = max(fused_diff, max(float(np.abs(x - y).max() / np.abs(y).max()) for x, y in zip(dens_f1, dens32)))
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
            "fp32_fused": {"value": cuf / tf, "unit": METRIC, "seconds": tf, "gpu_launches_approx": launches_f,
                           "form": "one launch of each substep kernel per ring width, the width lanes side by side, "
                                   "one graph per DT round, masked subcycling (fargo_batch_fuse)",
                           "speedup_over_per_disk_graphs": (cuf / tf) / v32,
                           "group_ms_per_substep": groups_ms,
                           "one_lane": {"value": cuf1 / tf1, "unit": METRIC, "seconds": tf1,
                                        "gpu_launches_approx": launches_f1,
                                        "form": "one launch of each substep kernel for the whole ensemble "
                                                "(fargo_batch_fuse_by_width(b, 0))",
                                        "speedup_over_per_disk_graphs": (cuf1 / tf1) / v32},
                           "dens_max_rel_diff_vs_per_disk": fused_diff},
            "fp64_plain_sequential": {"value": v64, "unit": METRIC, "seconds": t64},
            "fp64_batched": {"value": cu64b / t64b, "unit": METRIC, "seconds": t64b,
                             "form": "the same per-disk graphs side by side, FP64"},
            "ratio_fp32_batched_to_fp64_plain": v32 / v64,
            "ratio_fp32_batched_to_fp64_batched": v32 / (cu64b / t64b),
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
