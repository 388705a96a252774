"""CPU restatement of the learned correction's flux divergence, its adjoint and the
fine -> coarse restriction of its training targets (TEST INFRASTRUCTURE ONLY).

Only tests/ may import this module: it checks k_divergence, k_residual,
k_adjoint and k_restrict (cudaprotoplanetarydisks_gb300/csrc/fargo_learned.cu,
through fargo_learned_divergence / fargo_learned_loss / fargo_learned_restrict)
and is never the measured or shipped path.  The reference has no learned part; this restates the definition
the kernels implement, in FP64.

The outputs y[(i, j)] = (y_r, y_phi) are the mass fluxes (in units of
scale Surf_i) through the inner radial and the left azimuthal face of cell (i, j);
walls carry none (y_r of ring 0 and of ring nrad are taken as zero):
  dSigma(i, j) = scale [y_r(i, j) - y_r(i+1, j) Surf_{i+1} / Surf_i]
               + scale [y_phi(i, j) - y_phi(i, j+1)].
"""
import numpy as np


def divergence(y, surf, nrad, nsec, scale):
    y = np.asarray(y, dtype=np.float64).reshape(nrad, nsec, 2)
    s = np.asarray(surf, dtype=np.float64)[:nrad]
    yr = y[:, :, 0].copy()
    yr[0] = 0.0
    yr_next = np.zeros_like(yr)
    yr_next[:-1] = yr[1:] * (s[1:] / s[:-1])[:, None]
    yp = y[:, :, 1]
    return (scale * ((yr - yr_next) + (yp - np.roll(yp, -1, axis=1)))).ravel()


def adjoint(e, surf, nrad, nsec, scale):
    """dL/dy for dL/d(dSigma) = e: the transpose of divergence."""
    e = np.asarray(e, dtype=np.float64).reshape(nrad, nsec)
    s = np.asarray(surf, dtype=np.float64)[:nrad]
    gr = np.zeros_like(e)
    gr[1:] = scale * (e[1:] - e[:-1] * (s[1:] / s[:-1])[:, None])
    gp = scale * (e - np.roll(e, 1, axis=1))
    return np.stack([gr, gp], axis=-1).reshape(nrad * nsec, 2)


def loss(y, target, surf, nrad, nsec, scale, inv_var):
    """(dSigma, sum (dSigma - target)^2, dL/dy) for L = that sum * inv_var / n."""
    n = nrad * nsec
    ds = divergence(y, surf, nrad, nsec, scale)
    r = ds - np.asarray(target, dtype=np.float64)
    e = 2.0 * inv_var / n * r
    return ds, float((r * r).sum()), adjoint(e, surf, nrad, nsec, scale)


def restrict(fd, fvr, fvt, fsurf, factor):
    """The training targets' fine -> coarse restriction by `factor` (k_restrict):
    density area-weighted over the fine cells of a coarse cell; the radial
    velocity of coarse interface i = mean over its F fine sectors of fine interface
    F i; the azimuthal velocity of coarse face j = the fine face F j, weighted by
    the fine rings' surfaces; the ghost ring from the fine ghost ring (means over
    the F sectors).  Fine fields: [F nrad + 1, F nsec].  Returns coarse
    (dens, vrad, vtheta), [nrad + 1, nsec] each."""
    F = factor
    fd, fvr, fvt = (np.asarray(a, dtype=np.float64) for a in (fd, fvr, fvt))
    fnrad, fnsec = fd.shape[0] - 1, fd.shape[1]
    nrad, nsec = fnrad // F, fnsec // F
    sf = np.asarray(fsurf, dtype=np.float64)[:fnrad]
    w = sf.reshape(nrad, F)
    d = (fd[:fnrad].reshape(nrad, F, nsec, F) * w[:, :, None, None]).sum(axis=(1, 3)) / (F * w.sum(axis=1))[:, None]
    vt = (fvt[:fnrad, ::F].reshape(nrad, F, nsec) * w[:, :, None]).sum(axis=1) / w.sum(axis=1)[:, None]
    vr = fvr[::F].reshape(nrad + 1, nsec, F).mean(axis=2)
    ghost = lambda a: a[fnrad].reshape(nsec, F).mean(axis=1)  # noqa: E731
    dens = np.vstack([d, ghost(fd)])
    vtheta = np.vstack([vt, ghost(fvt)])
    return dens, vr, vtheta
