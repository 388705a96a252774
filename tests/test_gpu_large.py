"""The reference's largest grids (in/template4.par: 2048 x 4096, in/temp.par:
4096 x 4096; adiabatic, non-reflecting inner boundary, guiding-center frame, one
Jupiter-mass planet, no self-gravity), too large for the CPU oracle: checked by
properties that hold at any size.  At 4096 sectors the step takes its
wide-ring forms (the streamed CFL kernel; the register azimuthal transport with
several chunks of four cells per thread in FP32, the barrier-per-phase one with
global-memory ring buffers in FP64)."""
import os

import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from tests.helpers import rel_l2, small

pytestmark = pytest.mark.gpu

SIZES = [(2048, 4096), (4096, 4096)]


def large(nrad, nsec):
    return small("c3", nrad=nrad, nsec=nsec, non_reflecting=1, corotating=1, guiding_center=1, cooling=0,
                 rmin=0.4, rmax=2.5)


def _disk(params, planets, prec, env=None):
    old = {k: os.environ.get(k) for k in (env or {})}
    os.environ.update(env or {})
    try:
        return fg.Disk(params, planets, prec)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


@pytest.mark.parametrize("nrad,nsec", SIZES)
def test_largest_grids_step_consistently(nrad, nsec):
    params, planets = large(nrad, nsec)
    d64 = _disk(params, planets, fg.FARGO_FP64)
    n64 = d64.step_DT()
    f64 = {k: d64.field(k) for k in ("dens", "vrad", "vtheta", "energy")}
    d64.close()
    d32 = _disk(params, planets, fg.FARGO_FP32_BULK)
    n32 = d32.step_DT()
    f32 = {k: d32.field(k) for k in ("dens", "vrad", "vtheta", "energy")}
    d32.close()
    assert n32 == n64 > 0
    for k in f64:
        assert np.isfinite(f64[k]).all() and np.isfinite(f32[k]).all(), k
    assert (f64["dens"][:-1] > 0).all() and (f64["energy"][:-1] > 0).all()
    for k in ("dens", "vtheta", "energy"):
        assert rel_l2(f32[k], f64[k]) < 1e-4, (k, rel_l2(f32[k], f64[k]))


def test_wide_ring_transport_paths_agree():
    # 4096 FP32 sectors: the register kernel in chunks of four cells (several per
    # thread) against the barrier-per-phase kernel, whose shared- and global-memory
    # ring buffers agree bitwise.  The two kernels sum the ring mean in different
    # orders, so they differ by FP32 rounding: less than either differs from the
    # FP64 step, and the register kernel is as close to FP64 as the other one
    params, planets = large(*SIZES[0])
    names = ("dens", "vrad", "vtheta", "energy")

    def fields(prec, env=None):
        d = _disk(params, planets, prec, env)
        n = d.step_DT()
        f = {k: d.field(k) for k in names}
        d.close()
        return n, f

    n64, f64 = fields(fg.FARGO_FP64)
    nr, reg = fields(fg.FARGO_FP32_BULK)
    ng, gen = fields(fg.FARGO_FP32_BULK, {"FARGO_AZ_GENERIC": "1"})
    nb, glo = fields(fg.FARGO_FP32_BULK, {"FARGO_AZ_GLOBAL": "1"})
    assert n64 == nr == ng == nb
    for k in names:
        assert np.array_equal(gen[k], glo[k]), k
        e_rg, e_g64, e_r64 = rel_l2(reg[k], gen[k]), rel_l2(gen[k], f64[k]), rel_l2(reg[k], f64[k])
        assert e_rg < 0.5 * e_g64, (k, e_rg, e_g64)
        assert e_r64 < 1.1 * e_g64, (k, e_r64, e_g64)
