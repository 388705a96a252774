"""FP32-bulk drift against FP64 over long runs.

The same disk is advanced in the FP64 mode and in the FP32-bulk mode from the same
initial state, DT by DT, and after every `every` orbits of the planet the relative
L2 and Linf differences of the density (and of v_r, v_theta) are recorded.  An
orbit of a planet at r = 1 is 2 pi time units; at DT = 0.314159265359 (the
workloads' DT) 100 orbits are 2000 DTs.

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


def drift(cfg="c2", orbits=100, every=10, period=2.0 * math.pi, disk=None, **overrides):
    """Runs `orbits` planet orbits of workload `cfg` (or of disk = (params,
    planets)) in FP64 and FP32-bulk; returns the per-field relative differences
    after every `every` orbits."""
    params, planets = disk if disk is not None else load_config(cfg, **overrides)
    per_orbit = period / params.dt
    d64 = Disk(params, planets, FARGO_FP64)
    d32 = Disk(params, planets, FARGO_FP32_BULK)
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
            ndt = target
            row = {"orbits": k, "dts": ndt}
            for name in ("dens", "vrad", "vtheta"):
                l2, linf = _rel(d32.field(name), d64.field(name))
                row[name] = {"rel_l2": l2, "rel_linf": linf}
            rows.append(row)
        s64, s32 = d64.scalars(), d32.scalars()
        return {"workload": cfg, "nrad": params.nrad, "nsec": params.nsec, "orbits": orbits,
                "dts": ndt, "substeps_fp64": s64.substeps, "substeps_fp32": s32.substeps,
                "seconds_fp64": t64, "seconds_fp32": t32, "by_orbit": rows,
                "final_dens_rel_l2": rows[-1]["dens"]["rel_l2"]}
    finally:
        d64.close()
        d32.close()


if __name__ == "__main__":
    cfg = sys.argv[1] if len(sys.argv) > 1 else "c2"
    orbits = int(sys.argv[2]) if len(sys.argv) > 2 else 100
    print(json.dumps(drift(cfg, orbits)))
