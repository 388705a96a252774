"""CPU restatement of the learned correction's stencil MLP (TEST INFRASTRUCTURE ONLY).

Only tests/ may import this module: it checks the GPU kernels of
cudaprotoplanetarydisks_gb300/csrc/fargo_mlp.cu and is never the measured or
shipped path.  The network has no counterpart in the reference (the reference has
no learned part); this file restates the design the kernels implement:

    z1 = bf16(x W1 + b1), h1 = bf16(gelu(z1)), z2 = bf16(h1 W2 + b2),
    h2 = bf16(gelu(z2)), y = h2 W3[:, :2] + b3[:2]

with GELU in its tanh form z (1 + tanh u) / 2, u = sqrt(2/pi) (z + 0.044715 z^3)
(Hendrycks & Gimpel 2016), BF16 weights and inputs, sums in FP64 (the kernels accumulate in FP32), and
the backward pass with the kernels' rounding points (dy, dz2, dz1 rounded to
BF16).  `exact=True` drops every rounding: the plain FP64 network, whose
gradient the tests check against finite differences.
"""
import math

import numpy as np

NIN, NH, NOUT, NOUTP = 128, 64, 2, 8
OFF_W1 = 0
OFF_B1 = OFF_W1 + NIN * NH
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH * NOUTP
NPARAM = OFF_B3 + NOUTP


def bf16(x):
    """Round to BF16 (round to nearest even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


def _sig(z):
    """sigma(2u), u = sqrt(2/pi) (z + 0.044715 z^3): GELU in its tanh form
    (Hendrycks & Gimpel 2016), z (1 + tanh u) / 2 = z sigma(2u)."""
    u2 = 2.0 * math.sqrt(2.0 / math.pi) * (z + 0.044715 * z ** 3)
    return 0.5 * (1.0 + np.tanh(0.5 * u2))


def gelu(z):
    return z * _sig(z)


def gelu_d(z):
    s = _sig(z)
    return s + z * s * (1.0 - s) * 2.0 * math.sqrt(2.0 / math.pi) * (1.0 + 3.0 * 0.044715 * z * z)


def unpack(P, exact=False):
    P = np.asarray(P, dtype=np.float64)
    r = (lambda v: v) if exact else bf16
    W1 = r(P[OFF_W1:OFF_B1].reshape(NIN, NH))
    W2 = r(P[OFF_W2:OFF_B2].reshape(NH, NH))
    W3 = r(P[OFF_W3:OFF_B3].reshape(NH, NOUTP)[:, :NOUT])
    b1, b2, b3 = P[OFF_B1:OFF_W2], P[OFF_B2:OFF_W3], P[OFF_B3:OFF_B3 + NOUT]
    return W1, b1, W2, b2, W3, b3


def forward(P, X, exact=False):
    """y [n, 2] and the cache of the backward pass; X [n, 128] (BF16 values
    unless exact)."""
    r = (lambda v: v) if exact else bf16
    W1, b1, W2, b2, W3, b3 = unpack(P, exact)
    X = np.asarray(X, dtype=np.float64)
    z1 = r(X @ W1 + b1)
    h1 = r(gelu(z1))
    z2 = r(h1 @ W2 + b2)
    h2 = r(gelu(z2))
    y = h2 @ W3 + b3
    return y, (X, z1, h1, z2, h2)


def backward(P, cache, dy, exact=False):
    """Gradient blob (NPARAM) of sum(dy * y)."""
    r = (lambda v: v) if exact else bf16
    W1, b1, W2, b2, W3, b3 = unpack(P, exact)
    X, z1, h1, z2, h2 = cache
    dyb = r(np.asarray(dy, dtype=np.float64))
    dz2 = r((dyb @ W3.T) * gelu_d(z2))
    dz1 = r((dz2 @ W2.T) * gelu_d(z1))
    g = np.zeros(NPARAM)
    g[OFF_W1:OFF_B1] = (X.T @ dz1).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W2:OFF_B2] = (h1.T @ dz2).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    w3 = np.zeros((NH, NOUTP))
    w3[:, :NOUT] = h2.T @ dyb
    g[OFF_W3:OFF_B3] = w3.ravel()
    g[OFF_B3:OFF_B3 + NOUT] = dyb.sum(0)
    return g
