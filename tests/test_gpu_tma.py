"""The radial transport with TMA-staged tiles (k_transport_radial_tma) against the
same transport with per-thread loads (k_transport_radial, FARGO_NO_TMA=1).

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
    old = os.environ.get("FARGO_NO_TMA")
    if no_tma:
        os.environ["FARGO_NO_TMA"] = "1"
    else:
        os.environ.pop("FARGO_NO_TMA", None)
    try:
        d = fg.Disk(params, planets, prec)
    finally:
        if old is None:
            os.environ.pop("FARGO_NO_TMA", None)
        else:
            os.environ["FARGO_NO_TMA"] = old
    n = [d.step_DT() for _ in range(ndt)]
    out = {k: d.field(k) for k in ("dens", "vrad", "vtheta", "energy")}
    s = d.scalars()
    d.close()
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
