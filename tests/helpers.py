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


def sg_direct_sum(params, rinf, rmed, dens):
    """Self-gravity accelerations of a disk as a direct O(N^2) sum, no FFT.

    The log-polar kernels of compute_kernel (src/SgMain.cu:49-81, its cosh in
    single precision as there), the packing of ComputeFFTKernel (src/Kernels.cu:
    858-861: S_r = Sigma sqrt(r/r0), S_theta = S_r r/r0), the product with -G of
    ComputeConvolutionKernel (src/Kernels.cu:871-889) as a circular convolution
    over 2 nrad rings (the upper half of S is zero) and nsec sectors, and the
    normalisation and self term of ComputeSgAccKernel (src/Kernels.cu:893-911).
    Returns (accr, acct) on rings 0..nrad-1.
    """
    import math
    n, m = params.nrad, params.nsec
    dens = np.asarray(dens)[:n]
    eps = params.thicknesssmoothing * params.aspectratio
    rstep = math.log(rinf[n] / rinf[0]) / n
    tstep = 2 * math.pi / m
    i = np.arange(2 * n)
    u = np.where(i < n, np.log(rinf[np.minimum(i, n)] / rinf[0]), -np.log(rinf[np.clip(2 * n - i, 0, n)] / rinf[0]))
    uu, tt = u[:, None], (2 * math.pi * np.arange(m) / m)[None, :]
    base = eps * eps * np.exp(uu) + 2.0 * (np.cosh(uu.astype(np.float32)).astype(np.float64) - np.cos(tt))
    kr = (1.0 + eps * eps - np.cos(tt) * np.exp(-uu)) * base ** -1.5
    kt = np.sin(tt) * base ** -1.5
    div = (rmed[:n] / rmed[0])[:, None]
    sr = dens * np.sqrt(div)
    st = sr * div
    gr = np.zeros((n, m))
    gt = np.zeros((n, m))
    for k in range(n):
        for l in range(m):
            gr += np.roll(np.roll(kr, k, axis=0), l, axis=1)[:n] * sr[k, l]
            gt += np.roll(np.roll(kt, k, axis=0), l, axis=1)[:n] * st[k, l]
    accr = -gr * rstep * tstep / np.sqrt(div) + dens * rstep * tstep / eps
    acct = -gt * rstep * tstep / (div * np.sqrt(div))
    return accr, acct


def lbp_profile(r, tau, nu, mass=1.0, r0=1.0):
    """Lynden-Bell & Pringle (1974) spreading ring: Sigma(x, tau) = (M / (pi R0^2))
    tau^-1 x^-1/4 exp(-(1 + x^2) / tau) I_1/4(2 x / tau), x = r / R0, tau = 12 nu t / R0^2."""
    import math
    from scipy.special import ive
    x = r / r0
    z = 2 * x / tau
    # I_1/4(z) exp(-(1 + x^2)/tau) = ive(z) exp(z - (1 + x^2)/tau) = ive(z) exp(-(1 - x)^2 / tau)
    return mass / (math.pi * r0 ** 2) / tau * x ** -0.25 * np.exp(-(1 - x) ** 2 / tau) * ive(0.25, z)


def _massless_planet(cfg, **kw):
    from cudaprotoplanetarydisks_gb300.config import set_planet_mass
    params, planets = fg.load_config(cfg, **kw)
    set_planet_mass(params, planets[0], 0.0)
    return params, planets


def rest_state(make):
    """One orbit of the c1 disk without viscosity, noise or planet mass, from
    make(params, planets) (an FP64 disk with field / step_DT / close).  Returns
    (max |dSigma| / max Sigma, max |v_r| of the inner interfaces, the largest
    departure from axisymmetry relative to max Sigma, c_s / v_K)."""
    import math
    params, planets = _massless_planet("c1", sigma_noise=0.0, viscosity=0.0)
    disk = make(params, planets)
    try:
        s0 = disk.field("dens")[:-1].copy()
        for _ in range(int(round(2 * math.pi / params.dt))):
            disk.step_DT()
        s1 = disk.field("dens")[:-1]
        vr = disk.field("vrad")[1:-1]
        return (float(np.abs(s1 - s0).max() / np.abs(s0).max()), float(np.abs(vr).max()),
                float(np.abs(s1 - s1.mean(axis=1, keepdims=True)).max() / np.abs(s1).max()), params.aspectratio)
    finally:
        disk.close()


def lbp_ring(make, nu=1e-4, tau0=0.016, tau1=0.032):
    """A Lynden-Bell & Pringle ring (constant nu, aspect ratio 1e-3, 256 x 384 on
    [0.4, 2.5], WALL boundaries) started from the solution at tau0 -- Keplerian
    rotation, v_r = -3 / (Sigma r^1/2) d(nu Sigma r^1/2) / dr at the interfaces --
    and advanced whole DTs to about tau1.  Returns (relative L2 error of the ring
    means against the solution where it exceeds 1e-3 of its peak, relative mass
    change, DTs, reached tau)."""
    params, planets = _massless_planet("c1", sigma_noise=0.0, viscosity=nu, aspectratio=1e-3, nrad=256, nsec=384,
                                       rmin=0.4, rmax=2.5)
    disk = make(params, planets)
    try:
        rinf, rmed, rsup, surf = disk.mesh()
        n, ns = params.nrad, params.nsec
        sig = np.zeros((n + 1, ns))
        sig[:n] = lbp_profile(rmed[:n], tau0, nu)[:, None]
        floor = 1e-10 * sig.max()
        sig[:n] += floor
        ri = rinf[:n]
        h = 1e-6
        g = lambda r: nu * (lbp_profile(r, tau0, nu) + floor) * np.sqrt(r)  # noqa: E731
        vr_i = -3.0 / ((lbp_profile(ri, tau0, nu) + floor) * np.sqrt(ri)) * (g(ri * (1 + h)) - g(ri * (1 - h))) / (2 * h * ri)
        vr = np.zeros((n + 1, ns))
        vr[1:n] = vr_i[1:, None]  # the wall rings keep v_r = 0
        vt = np.zeros((n + 1, ns))
        vt[:n] = (rmed[:n] ** -0.5)[:, None]
        disk.set_fields(dens=sig, vrad=vr, vtheta=vt)
        m0 = float((disk.field("dens")[:n] * surf[:n, None]).sum())
        ndt = int(round((tau1 - tau0) / (12 * nu) / params.dt))
        for _ in range(ndt):
            disk.step_DT()
        tau = tau0 + 12 * nu * ndt * params.dt
        got = disk.field("dens")[:n].mean(axis=1) - floor
        ref = lbp_profile(rmed[:n], tau, nu)
        m1 = float((disk.field("dens")[:n] * surf[:n, None]).sum())
        mask = ref > 1e-3 * ref.max()
        return float(np.linalg.norm((got - ref)[mask]) / np.linalg.norm(ref[mask])), abs(m1 - m0) / m0, ndt, tau
    finally:
        disk.close()
