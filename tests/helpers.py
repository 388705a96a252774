"""Shared helpers of the test suite (comparison metrics and workload set-up)."""
import numpy as np

import cudaprotoplanetarydisks_gb300 as fg


def rel_linf(a, b):
    """max |a - b| / max |b| over rings 0..nrad-1 (the dumped part of a field)."""
    a, b = np.asarray(a)[:-1], np.asarray(b)[:-1]
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / den) if den > 0 else float(np.abs(a - b).max())


def rel_l2(a, b):
    a, b = np.asarray(a)[:-1], np.asarray(b)[:-1]
    den = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / den) if den > 0 else float(np.linalg.norm(a - b))


def small(cfg, nrad=64, nsec=192, **kw):
    return fg.load_config(cfg, nrad=nrad, nsec=nsec, **kw)


def disk_mass(fields_dens, surf):
    return float((np.asarray(fields_dens)[:-1] * np.asarray(surf)[:-1, None]).sum())
