"""The radial transport with TMA-staged tiles (k_transport_radial_tma) against the
same transport with per-thread loads (k_transport_radial, FARGO_NO_TMA=1), and the
column march (k_transport_radial_col, variant rad_col) against both.

Both form every cell from the same inputs with the same arithmetic; only the way
the tile reaches shared memory differs (cp.async.bulk.tensor into a double-buffered
stage of a persistent CTA, zero fill outside the field).  So whole DTs must agree
bitwise, in both precisions, with partial tiles in both directions (nsec not a
multiple of 32, nrad not a multiple of 16), with the energy equation, and with an
open inner boundary (whose lost mass the radial update records).  Rows whose byte
stride is not a multiple of 16 take the per-thread kernel.
"""
import os

import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from tests.helpers import small

pytestmark = pytest.mark.gpu

CASES = [
    ("c1", fg.FARGO_FP64, 64, 192, {}),
    ("c1", fg.FARGO_FP32_BULK, 72, 200, {}),
    ("c3", fg.FARGO_FP64, 40, 100, {}),
    ("c3", fg.FARGO_FP32_BULK, 56, 228, {}),
    ("c1", fg.FARGO_FP64, 48, 136, {"open_inner": 1}),
    ("c1", fg.FARGO_FP32_BULK, 48, 98, {}),  # 392-byte rows: the per-thread kernel
]


def run(params, planets, prec, ndt, no_tma):
    v = fg.default_variant()
    v.rad_col = 0  # the tile forms (FP32-bulk would take the column march by default)
    v.rad_tma = 0 if no_tma else 1
    b = fg.Batch([(params, planets)], prec, variant=v)
    d = b.disk(0)
    n = [d.step_DT() for _ in range(ndt)]
    out = {k: d.field(k) for k in ("dens", "vrad", "vtheta", "energy")}
    s = d.scalars()
    b.close()
    return n, out, s


@pytest.mark.parametrize("cfg,prec,nrad,nsec,extra", CASES)
def test_tma_radial_transport_is_bitwise_the_plain_one(cfg, prec, nrad, nsec, extra):
    params, planets = small(cfg, nrad=nrad, nsec=nsec)
    for k, v in extra.items():
        setattr(params, k, v)
    n1, f1, s1 = run(params, planets, prec, 2, no_tma=False)
    n0, f0, s0 = run(params, planets, prec, 2, no_tma=True)
    assert n1 == n0
    for k in f0:
        assert np.array_equal(f1[k], f0[k]), k
    assert s1.lost_mass == s0.lost_mass


def test_tma_kernel_is_the_one_launched():
    params, planets = small("c3", nrad=40, nsec=128)
    d = fg.Disk(params, planets, fg.FARGO_FP64)
    import ctypes
    ms = (ctypes.c_double * 96)()
    nk = ctypes.c_int(0)
    assert d.lib.fargo_time_substep_kernels(d.h, 1, ms, 96, ctypes.byref(nk)) == 0
    names = [d.lib.fargo_substep_kernel_name(d.h, k).decode() for k in range(nk.value)]
    d.close()
    assert "k_transport_radial_tma" in names and "k_transport_radial" not in names


def run_variant(params, planets, prec, ndt, **fields):
    v = fg.default_variant()
    for k, x in fields.items():
        setattr(v, k, x)
    b = fg.Batch([(params, planets)], prec, variant=v)
    d = b.disk(0)
    n = [d.step_DT() for _ in range(ndt)]
    out = {k: d.field(k) for k in ("dens", "vrad", "vtheta", "energy")}
    s = d.scalars()
    b.close()
    return n, out, s


@pytest.mark.parametrize("cfg,prec,nrad,nsec,extra", CASES)
def test_column_march_radial_transport(cfg, prec, nrad, nsec, extra):
    # the column march forms every cell with the tile kernel's arithmetic in the
    # same order: FP32 fields are bitwise the tile kernel's; FP64 (out-of-line
    # bodies, compiled apart from the tile kernel's) within rounding
    params, planets = small(cfg, nrad=nrad, nsec=nsec)
    for k, v in extra.items():
        setattr(params, k, v)
    n1, f1, s1 = run_variant(params, planets, prec, 2, rad_col=1)
    n0, f0, s0 = run_variant(params, planets, prec, 2, rad_col=0)
    assert n1 == n0
    for k in f0:
        if prec == fg.FARGO_FP32_BULK:
            assert np.array_equal(f1[k], f0[k]), k
        else:
            scale = max(float(np.abs(f0[k]).max()), 1e-300)
            assert float(np.abs(f1[k] - f0[k]).max()) <= 1e-13 * scale, k
    if prec == fg.FARGO_FP32_BULK:
        assert s1.lost_mass == s0.lost_mass
