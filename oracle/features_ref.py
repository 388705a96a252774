"""CPU restatement of the learned correction's input features (TEST INFRASTRUCTURE ONLY).

Only tests/ may import this module: it checks k_features
(cudaprotoplanetarydisks_gb300/csrc/fargo_learned.cu) and is never the measured
or shipped path.  The reference has no learned part; this file restates the
feature definition the kernel implements, in FP64:

per coarse cell (i, j) and neighbour (i + di, j + dj), di, dj in -2..2 (rings
clamped at the edges, sectors periodic), five channels:
  0  Sigma / Sigma(i, j) - 1            (centre: log Sigma(i, j))
  1  cell-centred v_r                    (mean of the cell's two interface values)
  2  cell-centred v_theta - the centre's (centre: v_theta - Rmed^-1/2)
  3  log Rmed - log Rmed(i)              (centre: log Rmed(i))
  4  azimuth of the cell centre from the first planet, over pi, in [-1, 1)
feature ((di + 2) * 5 + (dj + 2)) * 5 + ch, normalised as (v - mean) / std;
features 125..127 are zero.
"""
import math

import numpy as np


def features(dens, vrad, vtheta, rmed, phi_planet, norm=None):
    """dens, vrad, vtheta: [nrad + 1, nsec] fields; rmed: nrad + 1 radii.
    norm: 125 means then 125 deviations (None: identity).  Returns [nrad * nsec, 128]."""
    nrad, nsec = dens.shape[0] - 1, dens.shape[1]
    d = np.asarray(dens, dtype=np.float64)
    vr = np.asarray(vrad, dtype=np.float64)
    vt = np.asarray(vtheta, dtype=np.float64)
    rm = np.asarray(rmed, dtype=np.float64)[:nrad]
    vr_c = 0.5 * (vr[:nrad] + vr[1:nrad + 1])
    vt_c = 0.5 * (vt[:nrad] + np.roll(vt[:nrad], -1, axis=1))
    dphi = 2.0 * math.pi / nsec
    ang = (np.arange(nsec) + 0.5) * dphi - phi_planet
    ang = ang - 2.0 * math.pi * np.floor(ang / (2.0 * math.pi) + 0.5)
    ii, jj = np.meshgrid(np.arange(nrad), np.arange(nsec), indexing="ij")
    d0 = d[:nrad]
    out = np.zeros((nrad, nsec, 128))
    for di in range(-2, 3):
        ri = np.clip(ii + di, 0, nrad - 1)
        for dj in range(-2, 3):
            rj = (jj + dj) % nsec
            base = ((di + 2) * 5 + (dj + 2)) * 5
            if di == 0 and dj == 0:
                v0 = np.log(d0)
                v2 = vt_c - rm[:, None] ** -0.5
                v3 = np.broadcast_to(np.log(rm)[:, None], (nrad, nsec))
            else:
                v0 = (d[ri, rj] - d0) / d0
                v2 = vt_c[ri, rj] - vt_c
                v3 = np.log(rm[ri]) - np.log(rm)[:, None]
            vals = (v0, vr_c[ri, rj], v2, v3, ang[rj] / math.pi)
            for ch, v in enumerate(vals):
                out[:, :, base + ch] = v
    out = out.reshape(nrad * nsec, 128)
    if norm is not None:
        norm = np.asarray(norm, dtype=np.float64)
        std = np.where(norm[125:] > 0, norm[125:], 1.0)
        out[:, :125] = (out[:, :125] - norm[:125]) / std
    return out
