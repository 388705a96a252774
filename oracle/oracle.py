"""ctypes wrapper of the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may import
this module; it is the checker, never the measured or shipped path.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from cudaprotoplanetarydisks_gb300._capi import (  # noqa: E402
    FIELDS, FargoParams, FargoPlanet, FargoScalars)

from . import build as _build  # noqa: E402

_D = ctypes.c_double
_DP = ctypes.POINTER(_D)
_lib = None


def load():
    global _lib
    if _lib is None:
        path = _build.build()
        lib = ctypes.CDLL(path)
        sig = [
            ("orc_create", ctypes.c_void_p, [ctypes.POINTER(FargoParams), ctypes.POINTER(FargoPlanet), ctypes.c_int]),
            ("orc_destroy", None, [ctypes.c_void_p]),
            ("orc_last_error", ctypes.c_char_p, [ctypes.c_void_p]),
            ("orc_set_threads", None, [ctypes.c_int]),
            ("orc_get_threads", ctypes.c_int, []),
            ("orc_get_field", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _DP]),
            ("orc_set_fields", ctypes.c_int, [ctypes.c_void_p, _DP, _DP, _DP, _DP]),
            ("orc_algogas", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
            ("orc_condition_cfl", ctypes.c_int, [ctypes.c_void_p, _D, ctypes.POINTER(ctypes.c_int)]),
            ("orc_substep_full", ctypes.c_int, [ctypes.c_void_p, _D]),
            ("orc_substep", ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, _D]),
            ("orc_get_planets", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FargoPlanet), ctypes.c_int,
                                               ctypes.POINTER(ctypes.c_int)]),
            ("orc_get_scalars", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FargoScalars)]),
            ("orc_get_mesh", ctypes.c_int, [ctypes.c_void_p, _DP, _DP, _DP, _DP]),
            ("orc_fft2d", ctypes.c_int, [_DP, ctypes.c_int, ctypes.c_int, ctypes.c_int]),
            ("orc_device_reduce", _D, [_DP, ctypes.c_int]),
        ]
        for name, res, args in sig:
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
    return _lib


def _ptr(a):
    return a.ctypes.data_as(_DP) if a is not None else None


class OracleDisk:
    """FP64 CPU restatement of the reference step (see oracle/fargo_oracle.cpp)."""

    def __init__(self, params, planets):
        lib = load()
        self.lib = lib
        self.params = params
        self.nrad, self.nsec = params.nrad, params.nsec
        arr = (FargoPlanet * max(1, len(planets)))(*planets)
        self.h = lib.orc_create(ctypes.byref(params), arr, len(planets))
        if not self.h:
            raise RuntimeError("oracle: invalid parameters")

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def set_threads(n):
        load().orc_set_threads(int(n))

    @staticmethod
    def threads():
        return load().orc_get_threads()

    def field(self, name):
        out = np.empty(((self.nrad + 1), self.nsec), dtype=np.float64)
        rc = self.lib.orc_get_field(self.h, FIELDS[name], _ptr(out))
        if rc:
            raise RuntimeError(f"oracle field {name}: rc={rc}")
        return out

    def set_fields(self, dens=None, vrad=None, vtheta=None, energy=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (dens, vrad, vtheta, energy)]
        self.lib.orc_set_fields(self.h, *[_ptr(a) for a in arrs])

    def step_DT(self):
        n = ctypes.c_int(0)
        rc = self.lib.orc_algogas(self.h, ctypes.byref(n))
        if rc:
            raise RuntimeError("oracle AlgoGas: " + self.lib.orc_last_error(self.h).decode())
        return n.value

    def substep_full(self, dt):
        self.lib.orc_substep_full(self.h, float(dt))

    def substep(self, which, dt):
        rc = self.lib.orc_substep(self.h, int(which), float(dt))
        if rc:
            raise RuntimeError(f"oracle substep {which}: rc={rc}")

    def condition_cfl(self, deltaT):
        c = ctypes.c_int(0)
        self.lib.orc_condition_cfl(self.h, float(deltaT), ctypes.byref(c))
        return c.value

    def planets(self):
        arr = (FargoPlanet * 64)()
        nb = ctypes.c_int(0)
        self.lib.orc_get_planets(self.h, arr, 64, ctypes.byref(nb))
        return [arr[k] for k in range(nb.value)]

    def scalars(self):
        s = FargoScalars()
        self.lib.orc_get_scalars(self.h, ctypes.byref(s))
        return s

    def mesh(self):
        n = self.nrad + 1
        rinf, rmed, rsup, surf = (np.empty(n) for _ in range(4))
        self.lib.orc_get_mesh(self.h, _ptr(rinf), _ptr(rmed), _ptr(rsup), _ptr(surf))
        return rinf, rmed, rsup, surf


def fft2d(a, sign):
    """Unnormalised 2D complex DFT of the oracle (cuFFT Z2Z convention)."""
    b = np.ascontiguousarray(a, dtype=np.complex128).copy()
    load().orc_fft2d(b.view(np.float64).ctypes.data_as(_DP), b.shape[0], b.shape[1], int(sign))
    return b


def device_reduce(x):
    x = np.ascontiguousarray(x, dtype=np.float64)
    return load().orc_device_reduce(_ptr(x), x.size)
