"""FP32-bulk drift against FP64 over long runs.

The same disk is advanced in the FP64 mode and in the FP32-bulk mode from the same
initial state, DT by DT, and after every `every` orbits of the planet the relative
L2 and Linf differences of the density (and of v_r, v_theta) are recorded.  An
orbit of a planet at r = 1 is 2 pi time units; at DT = 0.314159265359 (the
workloads' DT) 100 orbits are 2000 DTs.

With control=True a third disk runs beside them: the FP64 mode from the same
initial state with every density multiplied by 1 + 2^-52 u, u uniform in [-1, 1]
(a perturbation of one unit in the last place).  Its distance from the plain FP64
run is the growth that the disk itself gives to the smallest possible
perturbation; where the flow is unstable (a planet opening a gap, vortices at its
edges, a migrating planet), any two runs that are not bitwise equal -- FP64 with
another summation order as much as FP32 -- separate at that rate, and the
FP32-bulk distance cannot be told apart from it.

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
    dctl = None
    if control:
        dctl = Disk(params, planets, FARGO_FP64)
        dens = dctl.field("dens")
        u = np.random.default_rng(1).uniform(-1.0, 1.0, dens.shape)
        dctl.set_fields(dens=dens * (1.0 + u * 2.0 ** -52))
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
            if dctl is not None:
                dctl.run(n)
            ndt = target
            row = {"orbits": k, "dts": ndt}
            for name in ("dens", "vrad", "vtheta"):
                ref = d64.field(name)
                l2, linf = _rel(d32.field(name), ref)
                row[name] = {"rel_l2": l2, "rel_linf": linf}
                if dctl is not None:
                    l2c, linfc = _rel(dctl.field(name), ref)
                    row["control_" + name] = {"rel_l2": l2c, "rel_linf": linfc}
            rows.append(row)
        s64, s32 = d64.scalars(), d32.scalars()
        out = {"workload": cfg, "nrad": params.nrad, "nsec": params.nsec, "orbits": orbits,
               "dts": ndt, "substeps_fp64": s64.substeps, "substeps_fp32": s32.substeps,
               "seconds_fp64": t64, "seconds_fp32": t32, "by_orbit": rows,
               "final_dens_rel_l2": rows[-1]["dens"]["rel_l2"]}
        if dctl is not None:
            out["final_control_dens_rel_l2"] = rows[-1]["control_dens"]["rel_l2"]
        return out
    finally:
        d64.close()
        d32.close()
        if dctl is not None:
            dctl.close()

if __name__ == "__main__":
    cfg = sys.argv[1] if len(sys.argv) > 1 else "c2"
    orbits = int(sys.argv[2]) if len(sys.argv) > 2 else 100
    print(json.dumps(drift(cfg, orbits, control=True)))
