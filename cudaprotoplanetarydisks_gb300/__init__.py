"""GB300-native FARGO-ADSG 2D polar-grid hydro step (host-side Python API).

The compute path is libfargo_gb300.so (CUDA kernels for sm_103a behind the C-ABI
of include/fargo_gb300.h).  This module mirrors the reference's per-step entry
points (AlgoGas, Substep1/2/3, Transport, ConditionCFL, ...) on a Disk object;
it never computes anything itself and raises when the library is missing.
"""
import ctypes

import numpy as np

from . import _capi
from ._capi import (FARGO_FP32_BULK, FARGO_FP64, FIELDS, FORCE_LEVELS, SUB_BOUNDARY, SUB_ENERGY,  # noqa: F401
                    SUB_POTENTIAL, SUB_SOUNDSPEED, SUB_SOURCE, SUB_TEMPERATURE, SUB_TRANSPORT,
                    FargoParams, FargoPlanet, FargoScalars, FargoVariant)
from .config import c4_disks, default_params, load_config, read_par, read_planets  # noqa: F401

_DP = ctypes.POINTER(ctypes.c_double)


class FargoError(RuntimeError):
    pass


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_DP)


class Disk:
    """One disk on one GPU.  precision: FARGO_FP64 (parity mode) or FARGO_FP32_BULK."""

    def __init__(self, params, planets, precision=FARGO_FP64, stream=None, _handle=None):
        self.lib = _capi.load()
        self.params = params
        self.nrad, self.nsec = params.nrad, params.nsec
        self.precision = precision
        self.owned = _handle is None
        if _handle is not None:  # a disk of a Batch (owned by the batch)
            self.h = _handle
            return
        arr = (FargoPlanet * max(1, len(planets)))(*planets)
        h = ctypes.c_void_p()
        rc = self.lib.fargo_ctx_create(ctypes.byref(params), arr, len(planets), precision,
                                       ctypes.c_void_p(stream) if stream else None, ctypes.byref(h))
        if rc != _capi.FARGO_OK:
            raise FargoError(f"fargo_ctx_create failed with status {rc}")
        self.h = h

    def _check(self, rc, what):
        if rc != _capi.FARGO_OK:
            raise FargoError(f"{what}: status {rc}: {self.lib.fargo_last_error(self.h).decode()}")

    def close(self):
        if getattr(self, "h", None):
            if self.owned:
                self.lib.fargo_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state -------------------------------------------------------------
    def field(self, name):
        out = np.empty((self.nrad + 1, self.nsec), dtype=np.float64)
        self._check(self.lib.fargo_get_field(self.h, FIELDS[name], _ptr(out)), f"get_field({name})")
        return out

    def fields(self):
        return {k: self.field(k) for k in ("dens", "vrad", "vtheta", "energy", "temperature")}

    def set_fields(self, dens=None, vrad=None, vtheta=None, energy=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (dens, vrad, vtheta, energy)]
        self._check(self.lib.fargo_set_fields(self.h, *[_ptr(a) for a in arrs]), "set_fields")

    def planets(self):
        arr = (FargoPlanet * 64)()
        nb = ctypes.c_int(0)
        self._check(self.lib.fargo_get_planets(self.h, arr, 64, ctypes.byref(nb)), "get_planets")
        return [arr[k] for k in range(nb.value)]

    def scalars(self):
        s = FargoScalars()
        self._check(self.lib.fargo_get_scalars(self.h, ctypes.byref(s)), "get_scalars")
        return s

    def mesh(self):
        n = self.nrad + 1
        rinf, rmed, rsup, surf = (np.empty(n) for _ in range(4))
        self._check(self.lib.fargo_get_mesh(self.h, _ptr(rinf), _ptr(rmed), _ptr(rsup), _ptr(surf)), "get_mesh")
        return rinf, rmed, rsup, surf

    # -- stepping (reference entry points) ----------------------------------
    def step_DT(self):
        """AlgoGas: one DT; returns the number of hydro substeps."""
        n = ctypes.c_int(0)
        self._check(self.lib.fargo_step_DT(self.h, ctypes.byref(n)), "step_DT")
        return n.value

    def run(self, ndt):
        n = ctypes.c_longlong(0)
        self._check(self.lib.fargo_run(self.h, int(ndt), ctypes.byref(n)), "run")
        return n.value

    def run_async(self, ndt):
        self._check(self.lib.fargo_run_async(self.h, int(ndt)), "run_async")

    def sync(self):
        self._check(self.lib.fargo_sync(self.h), "sync")

    def substep_full(self, dt):
        self._check(self.lib.fargo_substep_full(self.h, float(dt)), "substep_full")

    def substep(self, which, dt):
        self._check(self.lib.fargo_substep(self.h, int(which), float(dt)), f"substep({which})")

    def condition_cfl(self, deltaT):
        c = ctypes.c_int(0)
        self._check(self.lib.fargo_condition_cfl(self.h, float(deltaT), ctypes.byref(c)), "condition_cfl")
        return c.value

    def write_outputs(self, index):
        self._check(self.lib.fargo_write_outputs(self.h, int(index)), "write_outputs")

    def write_dims(self):
        self._check(self.lib.fargo_write_dims(self.h), "write_dims")

    def restart(self, index):
        """Fields, planets and time of output `index` in the disk's OUTPUTDIR
        (fargo_restart)."""
        self._check(self.lib.fargo_restart(self.h, int(index)), "restart")

    def compute_force(self, x, y, smoothing, mass, a, rh):
        """The disk's force on (x, y) by inner/outer cells and Hill-cut level
        (fargo_compute_force): array [4, FORCE_LEVELS] = fx inner, fx outer,
        fy inner, fy outer."""
        out = (ctypes.c_double * (4 * FORCE_LEVELS))()
        self._check(self.lib.fargo_compute_force(self.h, x, y, smoothing, mass, a, rh, out), "compute_force")
        return np.array(out).reshape(4, FORCE_LEVELS)

    def update_log(self, timestep):
        """Appends the torque-log rows of every planet (fargo_update_log)."""
        self._check(self.lib.fargo_update_log(self.h, int(timestep)), "update_log")


def _batch_arrays(disks):
    n = len(disks)
    params = (FargoParams * n)(*[p for p, _ in disks])
    flat = [pl for _, pls in disks for pl in pls]
    planets = (FargoPlanet * max(1, len(flat)))(*flat)
    counts = (ctypes.c_int * n)(*[len(pls) for _, pls in disks])
    return params, planets, counts


def default_variant():
    """The default execution variant (with the FARGO_* switches applied)."""
    v = FargoVariant()
    _capi.load().fargo_variant_default(ctypes.byref(v))
    return v


def autotune(disks, precision=FARGO_FP32_BULK, ndt=2):
    """fargo_batch_autotune: the fastest execution variant of this ensemble, with
    its rate and the default's (cell-updates/s)."""
    params, planets, counts = _batch_arrays(disks)
    v = FargoVariant()
    best, dflt = ctypes.c_double(), ctypes.c_double()
    rc = _capi.load().fargo_batch_autotune(len(disks), params, planets, counts, precision, int(ndt), ctypes.byref(v),
                                          ctypes.byref(best), ctypes.byref(dflt))
    if rc != _capi.FARGO_OK:
        raise FargoError(f"fargo_batch_autotune: status {rc}")
    return v, best.value, dflt.value


class Batch:
    """An ensemble of independent disks (fargo_batch_*): each disk keeps its own
    fields, CFL step and DT graph; the batch runs the disks' graphs side by side.
    disks: a list of (params, planets); variant: a FargoVariant for every disk
    (None: the default), e.g. the one autotune() returns."""

    def __init__(self, disks, precision=FARGO_FP32_BULK, variant=None):
        self.lib = _capi.load()
        n = len(disks)
        params, planets, counts = _batch_arrays(disks)
        h = ctypes.c_void_p()
        rc = self.lib.fargo_batch_create_variant(n, params, planets, counts, precision,
                                                 ctypes.byref(variant) if variant is not None else None,
                                                 ctypes.byref(h))
        if rc != _capi.FARGO_OK:
            raise FargoError(f"fargo_batch_create failed with status {rc}")
        self.h = h
        self.disks = [Disk(p, [], precision, _handle=ctypes.c_void_p(self.lib.fargo_batch_disk(h, k)))
                      for k, (p, _) in enumerate(disks)]
        self.cells = sum(p.nrad * p.nsec for p, _ in disks)

    def __len__(self):
        return len(self.disks)

    def disk(self, k):
        return self.disks[k]

    def run_async(self, ndt):
        rc = self.lib.fargo_batch_run_async(self.h, int(ndt))
        if rc != _capi.FARGO_OK:
            raise FargoError(f"fargo_batch_run_async: status {rc}")

    def sync(self):
        rc = self.lib.fargo_batch_sync(self.h)
        if rc != _capi.FARGO_OK:
            raise FargoError(f"fargo_batch_sync: status {rc}")

    def fuse(self, by_width=True):
        """fargo_batch_fuse / fargo_batch_fuse_by_width: from now on every substep
        kernel runs once per lane of disks (one lane per ring width, or with
        by_width=False one for the whole ensemble; one graph per DT round, masked
        subcycling); raises with the reason when a disk uses a path the fused form
        does not carry."""
        rc = self.lib.fargo_batch_fuse_by_width(self.h, 1 if by_width else 0)
        if rc != _capi.FARGO_OK:
            raise FargoError(f"fargo_batch_fuse: status {rc}: {self.lib.fargo_batch_last_error(self.h).decode()}")
        return self

    def fused_lanes(self):
        n = ctypes.c_int(0)
        rc = self.lib.fargo_batch_fused_lanes(self.h, ctypes.byref(n))
        if rc != _capi.FARGO_OK:
            raise FargoError(f"fargo_batch_fused_lanes: status {rc}")
        return n.value

    def fused_kernel_times(self, reps=4):
        """[(kernel, mean ms)] of every launch group of one fused substep
        (fargo_batch_fused_time_kernels: starts a DT round, runs reps substeps)."""
        ms = (ctypes.c_double * 1024)()
        n = ctypes.c_int(0)
        rc = self.lib.fargo_batch_fused_time_kernels(self.h, reps, ms, 1024, ctypes.byref(n))
        if rc != _capi.FARGO_OK:
            raise FargoError(f"fargo_batch_fused_time_kernels: status {rc}")
        return [(self.lib.fargo_batch_fused_kernel_name(self.h, k).decode(), ms[k]) for k in range(n.value)]

    def fused_launches(self):
        """(launches per substep of the whole ensemble, launches per DT round)."""
        a, b = ctypes.c_int(0), ctypes.c_int(0)
        rc = self.lib.fargo_batch_fused_launches(self.h, ctypes.byref(a), ctypes.byref(b))
        if rc != _capi.FARGO_OK:
            raise FargoError(f"fargo_batch_fused_launches: status {rc}")
        return a.value, b.value

    def advance(self, t_end):
        """Every disk to physical time t_end (whole DTs of its own); returns the
        substeps of all disks."""
        n = ctypes.c_longlong(0)
        failed = ctypes.c_int(-1)
        rc = self.lib.fargo_batch_advance(self.h, float(t_end), ctypes.byref(n), ctypes.byref(failed))
        if rc != _capi.FARGO_OK:
            msg = self.lib.fargo_last_error(self.disks[failed.value].h).decode() if failed.value >= 0 else ""
            raise FargoError(f"fargo_batch_advance: status {rc} (disk {failed.value}): {msg}")
        return n.value

    def substeps(self):
        return sum(d.scalars().substeps for d in self.disks)

    def close(self):
        if getattr(self, "h", None):
            for d in self.disks:
                d.h = None
            self.lib.fargo_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
