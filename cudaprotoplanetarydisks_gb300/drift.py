"""FP32-bulk drift against FP64 over long runs.

The same disk is advanced in the FP64 mode and in the FP32-bulk mode from the same
initial state, DT by DT, and after every `every` orbits of the planet the relative
L2 and Linf differences of the density (and of v_r, v_theta) are recorded.  An
orbit of a planet at r = 1 is 2 pi time units; at DT = 0.314159265359 (the
workloads' DT) 100 orbits are 2000 DTs.

With control=True two more disks run beside them, both in the FP64 mode from the
same initial state with every density multiplied by 1 + e u, u uniform in
[-1, 1]: e = 2^-52 (one unit in the last place of FP64, "control") and e = 2^-24
(the rounding of an FP32 value, "control32").  Their distances from the plain
FP64 run show how the disk itself amplifies a perturbation of that size: where
the flow is unstable (a planet opening a gap, vortices at its edges, a migrating
planet), two runs that differ at the FP32 level separate whatever arithmetic
they use, and the FP32-bulk distance is then the flow's, not the arithmetic's.

    python -m cudaprotoplanetarydisks_gb300.drift [config] [orbits]
"""
import json
import math
import sys
import time

import numpy as np

from . import FARGO_FP32_BULK, FARGO_FP64, Disk, load_config


def _rel(a, b):
    a, b = a[:-1], b[:-1]
    return float(np.linalg.norm(a - b) / np.linalg.norm(b)), float(np.abs(a - b).max() / np.abs(b).max())


def drift(cfg="c2", orbits=100, every=10, period=2.0 * math.pi, disk=None, control=False, **overrides):
    """Runs `orbits` planet orbits of workload `cfg` (or of disk = (params,
    planets)) in FP64 and FP32-bulk (and, with control, FP64 from a one-ulp
    perturbed density); returns the per-field relative differences after every
    `every` orbits."""
    params, planets = disk if disk is not None else load_config(cfg, **overrides)
    per_orbit = period / params.dt
    d64 = Disk(params, planets, FARGO_FP64)
    d32 = Disk(params, planets, FARGO_FP32_BULK)
    controls = {}
    if control:
        for name, eps in (("control", 2.0 ** -52), ("control32", 2.0 ** -24)):
            d = Disk(params, planets, FARGO_FP64)
            dens = d.field("dens")
            u = np.random.default_rng(1).uniform(-1.0, 1.0, dens.shape)
            d.set_fields(dens=dens * (1.0 + u * eps))
            controls[name] = d
    rows, ndt, t64, t32 = [], 0, 0.0, 0.0
    try:
        for k in range(every, orbits + every, every):
            target = int(round(k * per_orbit))
            n = target - ndt
            t0 = time.perf_counter()
            d64.run(n)
            t64 += time.perf_counter() - t0
            t0 = time.perf_counter()
            d32.run(n)
            t32 += time.perf_counter() - t0
            for d in controls.values():
                d.run(n)
            ndt = target
            row = {"orbits": k, "dts": ndt}
            for name in ("dens", "vrad", "vtheta"):
                ref = d64.field(name)
                l2, linf = _rel(d32.field(name), ref)
                row[name] = {"rel_l2": l2, "rel_linf": linf}
                for cname, d in controls.items():
                    l2c, linfc = _rel(d.field(name), ref)
                    row[cname + "_" + name] = {"rel_l2": l2c, "rel_linf": linfc}
            rows.append(row)
        s64, s32 = d64.scalars(), d32.scalars()
        out = {"workload": cfg, "nrad": params.nrad, "nsec": params.nsec, "orbits": orbits,
               "dts": ndt, "substeps_fp64": s64.substeps, "substeps_fp32": s32.substeps,
               "seconds_fp64": t64, "seconds_fp32": t32, "by_orbit": rows,
               "final_dens_rel_l2": rows[-1]["dens"]["rel_l2"]}
        if controls:
            out["final_control_dens_rel_l2"] = rows[-1]["control_dens"]["rel_l2"]
            out["final_control32_dens_rel_l2"] = rows[-1]["control32_dens"]["rel_l2"]
        return out
    finally:
        d64.close()
        d32.close()
        for d in controls.values():
            d.close()

if __name__ == "__main__":
    cfg = sys.argv[1] if len(sys.argv) > 1 else "c2"
    orbits = int(sys.argv[2]) if len(sys.argv) > 2 else 100
    print(json.dumps(drift(cfg, orbits, control=True)))
