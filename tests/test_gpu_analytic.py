"""Analytic checks of the FP64 step, independent of the oracle.

Both hydro checks keep the planet file's planet with zero mass: the star's potential
enters the reference's potential together with the first planet
(FillForcesArrays / FillForcesArraysKernel, src/Pframeforce.cu:67-80,
src/Kernels.cu:1246-1251), so a disk with no planet at all feels no gravity.

* Rest state: a disk with a massless planet, no viscosity and no noise starts in the
  equilibrium the set-up builds (pressure-supported rotation, no radial flow) and
  stays there: over one orbit the density changes, and the radial velocity grows,
  only at the level of the discretisation error of that equilibrium.
* Viscous spreading of a ring (Lynden-Bell & Pringle 1974): with constant
  viscosity nu around a point mass and negligible pressure, a ring of surface
  density spreads as
      Sigma(x, tau) = (M / (pi R0^2)) tau^-1 x^-1/4 exp(-(1 + x^2) / tau) I_1/4(2 x / tau),
  x = r / R0, tau = 12 nu t / R0^2, with radial velocity
      v_r = -3 / (Sigma r^1/2) d(nu Sigma r^1/2) / dr.
  The disk starts from the solution at tau0 (Keplerian rotation, that v_r at the
  cell interfaces) and must reach the solution at tau1 within the resolution's
  error; its mass must be conserved to rounding (WALL boundaries, the ring far
  from them).
* Self-gravity: the FFT convolution against a direct sum of the same kernels.
* The ring and the self-gravity again in the FP32-bulk mode.
"""
import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from tests.helpers import lbp_ring, rest_state, sg_direct_sum

pytestmark = pytest.mark.gpu


def _fp64(params, planets):
    return fg.Disk(params, planets, fg.FARGO_FP64)


def test_rest_state_stays_steady():
    ds, vr_max, axi, cs = rest_state(_fp64)
    print(f"one orbit at rest: max |dSigma|/Sigma {ds:.2e}, max |v_r| {vr_max:.2e} (c_s/v_K = {cs})")
    # axisymmetric to rounding, and steady: the FP64 oracle gives 1.0e-3 and 1.0e-4
    # (the set-up's rotation balances the analytic pressure gradient, not the
    # discrete one)
    assert axi < 1e-12
    assert ds < 3e-3
    assert vr_max < 1e-2 * cs


def test_viscous_ring_spreading_matches_lynden_bell_pringle():
    pytest.importorskip("scipy")
    err, dm, ndt, tau = lbp_ring(_fp64)
    print(f"LBP ring to tau {tau:.4f} ({ndt} DTs): relative L2 {err:.2e}, mass change {dm:.1e}")
    # the FP64 oracle gives 8.3e-4 over these 42 DTs (262 substeps)
    assert dm <= 1e-12
    assert err < 5e-3


def test_self_gravity_matches_a_direct_convolution():
    # the FFT self-gravity of the initial 16 x 32 self-gravitating disk against the
    # direct sum of its kernels (the accelerations the set-up computes)
    params, planets = fg.load_config("c2", nrad=16, nsec=32)
    disk = fg.Disk(params, planets, fg.FARGO_FP64)
    try:
        rinf, rmed, _, _ = disk.mesh()
        accr, acct = sg_direct_sum(params, rinf, rmed, disk.field("dens"))
        n = params.nrad
        er = float(np.abs(disk.field("sg_accr")[:n] - accr).max() / np.abs(accr).max())
        et = float(np.abs(disk.field("sg_acct")[:n] - acct).max() / np.abs(acct).max())
    finally:
        disk.close()
    print(f"self-gravity against the direct sum: radial {er:.1e}, azimuthal {et:.1e}")
    # both take cosh in single precision; numpy's and the C library's may differ by an ulp
    assert er < 1e-6 and et < 1e-6


def test_fp32_bulk_viscous_ring_spreading():
    # the same ring in the FP32-bulk mode: the FP32 fields keep the analytic
    # solution's accuracy (the resolution's error dominates FP32 rounding)
    pytest.importorskip("scipy")
    err, dm, ndt, tau = lbp_ring(lambda p, pl: fg.Disk(p, pl, fg.FARGO_FP32_BULK))
    print(f"FP32-bulk LBP ring to tau {tau:.4f} ({ndt} DTs): relative L2 {err:.2e}, mass change {dm:.1e}")
    # measured 8.8e-4 (FP64: 8.3e-4) and a mass change of 8.6e-8 over the 42 DTs
    assert dm <= 1e-6
    assert err < 5e-3


def test_fp32_bulk_self_gravity_matches_a_direct_convolution():
    # the FP32-bulk self-gravity (FP32 FFTs, kernel spectra rounded from FP64)
    # against the same FP64 direct sum
    params, planets = fg.load_config("c2", nrad=16, nsec=32)
    disk = fg.Disk(params, planets, fg.FARGO_FP32_BULK)
    try:
        rinf, rmed, _, _ = disk.mesh()
        accr, acct = sg_direct_sum(params, rinf, rmed, disk.field("dens"))
        n = params.nrad
        er = float(np.abs(disk.field("sg_accr")[:n] - accr).max() / np.abs(accr).max())
        et = float(np.abs(disk.field("sg_acct")[:n] - acct).max() / np.abs(acct).max())
    finally:
        disk.close()
    print(f"FP32-bulk self-gravity against the direct sum: radial {er:.1e}, azimuthal {et:.1e}")
    # measured 2.0e-7 and 1.8e-4 (the azimuthal acceleration is the small one: the FP32
    # transforms' rounding relative to its maximum)
    assert er < 2e-6 and et < 2e-3
