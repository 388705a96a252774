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
