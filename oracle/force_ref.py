"""CPU restatement of the reference's disk-force diagnostics (TEST INFRASTRUCTURE ONLY).

Only tests/ may import this module: it checks fargo_compute_force and
fargo_update_log (cudaprotoplanetarydisks_gb300/csrc/fargo_force_diag.cu,
fargo_ctx.cu) and is never the measured or shipped path.  FP64 numpy; the
reference sums with DeviceReduce, here numpy sums (the orders differ: agreement
to roundoff, not bitwise).
"""
import math

import numpy as np

LEVELS = 11  # dimfxy, src/Main.cu:74


def compute_force(dens, rmed, surf, x, y, smoothing, a, rh, levels=LEVELS):
    """ComputeForce src/Force.cu:102-131 with ComputeForceKernel
    src/Kernels.cu:693-729.  dens: [nrad, nsec]; rmed, surf: the first nrad
    entries.  Returns GlobalForce as [4, levels]: fx inner, fx outer, fy inner,
    fy outer (inner: Rmed < a)."""
    nrad, nsec = dens.shape
    phi = 2.0 * np.pi * np.arange(nsec) / nsec  # CellAbscissa src/Kernels.cu:161-162
    cx = rmed[:nrad, None] * np.cos(phi)[None, :]
    cy = rmed[:nrad, None] * np.sin(phi)[None, :]
    cellmass = surf[:nrad, None] * dens
    dx, dy = cx - x, cy - y
    d2 = dx * dx + dy * dy
    dist2 = d2 + smoothing * smoothing
    inv3 = 1.0 / dist2 / np.sqrt(dist2)
    inner = (rmed[:nrad] < a)[:, None]
    out = np.zeros((4, levels))
    for k in range(levels):
        if k == 0:
            cut = 1.0
        else:
            rk = rh * (k / (levels - 1))
            cut = 1.0 - np.exp(-d2 / (rk * rk))
        fx = cellmass * dx * inv3 * cut
        fy = cellmass * dy * inv3 * cut
        out[0, k] = fx[np.broadcast_to(inner, fx.shape)].sum()
        out[1, k] = fx[~np.broadcast_to(inner, fx.shape)].sum()
        out[2, k] = fy[np.broadcast_to(inner, fy.shape)].sum()
        out[3, k] = fy[~np.broadcast_to(inner, fy.shape)].sum()
    return out


def torque_row(gf, x, y, vx, vy, t):
    """The nine values after TimeStep of a tqwk<k>.dat row, src/Force.cu:56-64."""
    fxi, fxei, fxo, fxeo = gf[0, 0], gf[0, -1], gf[1, 0], gf[1, -1]
    fyi, fyei, fyo, fyeo = gf[2, 0], gf[2, -1], gf[3, 0], gf[3, -1]
    return np.array([x * fyi - y * fxi, x * fyo - y * fxo, x * fyei - y * fxei, x * fyeo - y * fxeo,
                     vx * fxi + vy * fyi, vx * fxo + vy * fyo, vx * fxei + vy * fyei, vx * fxeo + vy * fyeo, t])


def hill_radius(m, a):
    """rh of UpdateLog, src/Force.cu:43."""
    return (m / 3.0) ** (1.0 / 3.0) * a + 1e-15


def direct_force(dens, rmed, surf, x, y, smoothing, a, rh, k, levels=LEVELS):
    """Plain loops over the cells for one level (pins compute_force on small grids)."""
    nrad, nsec = dens.shape
    f = [0.0, 0.0, 0.0, 0.0]
    for i in range(nrad):
        for j in range(nsec):
            m = surf[i] * dens[i, j]
            ang = 2.0 * math.pi * j / nsec
            dx = rmed[i] * math.cos(ang) - x
            dy = rmed[i] * math.sin(ang) - y
            d2 = dx * dx + dy * dy
            dist2 = d2 + smoothing * smoothing
            inv3 = 1.0 / dist2 / math.sqrt(dist2)
            cut = 1.0 if k == 0 else 1.0 - math.exp(-d2 / (rh * k / (levels - 1)) ** 2)
            o = 0 if rmed[i] < a else 1
            f[o] += m * dx * inv3 * cut
            f[2 + o] += m * dy * inv3 * cut
    return f
