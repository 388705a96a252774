"""Analytic checks of the FP64 step, independent of the oracle.

* Rest state: a disk without planet, viscosity or noise starts in the
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
"""
import math

import numpy as np
import pytest

import cudaprotoplanetarydisks_gb300 as fg
from tests.helpers import sg_direct_sum

pytestmark = pytest.mark.gpu


def test_rest_state_stays_steady():
    params, _ = fg.load_config("c1", sigma_noise=0.0, viscosity=0.0)
    disk = fg.Disk(params, [], fg.FARGO_FP64)
    try:
        s0 = disk.field("dens")[:-1].copy()
        cs = params.aspectratio  # cs / v_K
        orbit = int(round(2 * math.pi / params.dt))
        disk.run(orbit)
        s1 = disk.field("dens")[:-1]
        vr = disk.field("vrad")[1:-1]
        ds = float(np.abs(s1 - s0).max() / np.abs(s0).max())
        vr_max = float(np.abs(vr).max())
        print(f"one orbit at rest: max |dSigma|/Sigma {ds:.2e}, max |v_r| {vr_max:.2e} (c_s/v_K = {cs})")
        # axisymmetric to rounding, and steady to well below the sound speed's level
        assert float(np.abs(s1 - s1.mean(axis=1, keepdims=True)).max() / np.abs(s1).max()) < 1e-12
        assert ds < 1e-3
        assert vr_max < 1e-2 * cs
    finally:
        disk.close()


def _lbp(r, tau, nu, mass=1.0, r0=1.0):
    from scipy.special import ive
    x = r / r0
    z = 2 * x / tau
    # I_1/4(z) exp(-(1 + x^2)/tau) = ive(z) exp(z - (1 + x^2)/tau) = ive(z) exp(-(1 - x)^2 / tau)
    return mass / (math.pi * r0 ** 2) / tau * x ** -0.25 * np.exp(-(1 - x) ** 2 / tau) * ive(0.25, z)


def test_viscous_ring_spreading_matches_lynden_bell_pringle():
    pytest.importorskip("scipy")
    nu, tau0, tau1 = 1e-4, 0.016, 0.032
    params, _ = fg.load_config("c1", sigma_noise=0.0, viscosity=nu, aspectratio=1e-3, nrad=256, nsec=384,
                               rmin=0.4, rmax=2.5)
    disk = fg.Disk(params, [], fg.FARGO_FP64)
    try:
        rinf, rmed, rsup, surf = disk.mesh()
        n, ns = params.nrad, params.nsec
        sig = np.zeros((n + 1, ns))
        sig[:n] = _lbp(rmed[:n], tau0, nu)[:, None]
        floor = 1e-10 * sig.max()
        sig[:n] += floor
        # v_r at the interfaces r = rinf[i]: -3 / (Sigma r^1/2) d(nu Sigma r^1/2)/dr, from the solution
        ri = rinf[:n]
        h = 1e-6
        g = lambda r: nu * (_lbp(r, tau0, nu) + floor) * np.sqrt(r)  # noqa: E731
        vr_i = -3.0 / ((_lbp(ri, tau0, nu) + floor) * np.sqrt(ri)) * (g(ri * (1 + h)) - g(ri * (1 - h))) / (2 * h * ri)
        vr = np.zeros((n + 1, ns))
        vr[1:n] = vr_i[1:, None]  # the wall rings keep v_r = 0
        vt = np.zeros((n + 1, ns))
        vt[:n] = (rmed[:n] ** -0.5)[:, None]
        disk.set_fields(dens=sig, vrad=vr, vtheta=vt)
        m0 = float((disk.field("dens")[:n] * surf[:n, None]).sum())
        t1 = (tau1 - tau0) / (12 * nu)
        ndt = int(round(t1 / params.dt))
        disk.run(ndt)
        tau = tau0 + 12 * nu * ndt * params.dt
        got = disk.field("dens")[:n].mean(axis=1) - floor
        ref = _lbp(rmed[:n], tau, nu)
        m1 = float((disk.field("dens")[:n] * surf[:n, None]).sum())
        mask = ref > 1e-3 * ref.max()
        err = float(np.linalg.norm((got - ref)[mask]) / np.linalg.norm(ref[mask]))
        print(f"LBP ring, tau {tau0} -> {tau:.4f} ({ndt} DTs): relative L2 {err:.2e}, mass change {abs(m1 - m0) / m0:.1e}")
        assert abs(m1 - m0) <= 1e-12 * m0
        assert err < 0.05
    finally:
        disk.close()


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
