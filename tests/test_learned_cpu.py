"""The MLP oracle (oracle/mlp_ref.py) pinned on the CPU: its backward pass against
central finite differences of the exact FP64 network, and its BF16 rounding
against torch's."""
import numpy as np
import torch

from cudaprotoplanetarydisks_gb300.learned import NPARAM, init_params
from oracle import mlp_ref


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.normal(0, 1, 4000), rng.normal(0, 1e-3, 1000), [0.0, 1.0, -2.5, 65504.0, 1e-30]])
    ours = mlp_ref.bf16(x)
    ref = torch.tensor(x, dtype=torch.float32).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(ours, ref)


def test_oracle_gradient_matches_finite_differences():
    assert mlp_ref.NPARAM == NPARAM
    rng = np.random.default_rng(5)
    P = init_params(1).astype(np.float64)
    P[mlp_ref.OFF_B1:mlp_ref.OFF_W2] = rng.normal(0, 0.1, mlp_ref.NH)
    X = rng.normal(0, 1, (24, mlp_ref.NIN))
    dy = rng.normal(0, 1, (24, mlp_ref.NOUT))
    y, cache = mlp_ref.forward(P, X, exact=True)
    g = mlp_ref.backward(P, cache, dy, exact=True)

    def f(Q):
        return float((mlp_ref.forward(Q, X, exact=True)[0] * dy).sum())

    idx = list(rng.choice(np.arange(mlp_ref.OFF_W1, mlp_ref.OFF_B1), 12, replace=False)) + \
        list(rng.choice(np.arange(mlp_ref.OFF_W2, mlp_ref.OFF_B2), 8, replace=False)) + \
        [mlp_ref.OFF_B1 + 3, mlp_ref.OFF_B2 + 7, mlp_ref.OFF_W3 + 5 * mlp_ref.NOUTP + 1, mlp_ref.OFF_B3]
    h = 1e-6
    for p in idx:
        Qp, Qm = P.copy(), P.copy()
        Qp[p] += h
        Qm[p] -= h
        fd = (f(Qp) - f(Qm)) / (2 * h)
        assert abs(fd - g[p]) <= 1e-6 * max(1.0, abs(fd)), (p, fd, g[p])


def test_feature_oracle_layout():
    """oracle/features_ref.py against the definition, cell by cell, on a tiny grid."""
    from oracle import features_ref
    nrad, nsec = 5, 8
    rng = np.random.default_rng(0)
    d = 1.0 + 0.01 * rng.random((nrad + 1, nsec))
    vr, vt = rng.random((nrad + 1, nsec)), rng.random((nrad + 1, nsec))
    rm = np.linspace(1.0, 2.0, nrad + 1)
    f = features_ref.features(d, vr, vt, rm, 0.3)
    assert f.shape == (nrad * nsec, 128) and not f[:, 125:].any()
    i, j = 2, 3
    row = f[i * nsec + j]
    centre = (2 * 5 + 2) * 5
    assert np.isclose(row[centre], np.log(d[i, j])) and np.isclose(row[centre + 3], np.log(rm[i]))
    right = (2 * 5 + 3) * 5  # di = 0, dj = +1
    assert np.isclose(row[right], d[i, j + 1] / d[i, j] - 1)
    assert np.isclose(row[right + 1], 0.5 * (vr[i, j + 1] + vr[i + 1, j + 1]))
    vtc = lambda a, b: 0.5 * (vt[a, b] + vt[a, (b + 1) % nsec])  # noqa: E731
    assert np.isclose(row[right + 2], vtc(i, j + 1) - vtc(i, j)) and row[right + 3] == 0.0
    outer = (0 * 5 + 2) * 5  # di = -2 at ring 0 is clamped to ring 0
    row0 = f[0 * nsec + j]
    assert np.isclose(row0[outer], 0.0) and row0[outer + 3] == 0.0
    assert np.all(np.abs(f[:, 4::5][:, :25]) <= 1.0)


def test_flux_oracle_adjoint_and_mass():
    """oracle/flux_ref.py: the adjoint is the transpose (<D y, e> = <y, D^T e>), the
    divergence conserves mass (sum dSigma Surf = 0) and the loss gradient matches
    central finite differences."""
    from oracle import flux_ref
    rng = np.random.default_rng(9)
    nrad, nsec, scale = 6, 10, 0.7
    surf = np.linspace(1.0, 3.0, nrad + 1)
    y = rng.normal(0, 1, (nrad * nsec, 2))
    e = rng.normal(0, 1, nrad * nsec)
    ds = flux_ref.divergence(y, surf, nrad, nsec, scale)
    assert abs(np.dot(ds, e) - np.sum(y * flux_ref.adjoint(e, surf, nrad, nsec, scale))) < 1e-10
    assert abs((ds.reshape(nrad, nsec) * surf[:nrad, None]).sum()) < 1e-12
    target = rng.normal(0, 1, nrad * nsec)
    _, _, g = flux_ref.loss(y, target, surf, nrad, nsec, scale, 1.3)

    def f(yy):
        return flux_ref.loss(yy, target, surf, nrad, nsec, scale, 1.3)[1] * 1.3 / (nrad * nsec)

    for k in ((0, 0), (nsec + 3, 0), (17, 1), (nrad * nsec - 1, 1)):
        yp, ym = y.copy(), y.copy()
        yp[k] += 1e-6
        ym[k] -= 1e-6
        assert abs((f(yp) - f(ym)) / 2e-6 - g[k]) < 1e-7, k


def test_restriction_oracle_keeps_constants_and_mass():
    from oracle import flux_ref
    F, nrad, nsec = 4, 3, 5
    rng = np.random.default_rng(2)
    surf = np.linspace(1.0, 2.0, F * nrad + 1)
    const = np.full((F * nrad + 1, F * nsec), 2.0)
    d, vr, vt = flux_ref.restrict(const, -0.5 * const, 0.25 * const, surf, F)
    assert d.shape == vr.shape == vt.shape == (nrad + 1, nsec)
    assert np.allclose(d, 2.0) and np.allclose(vr, -1.0) and np.allclose(vt, 0.5)
    # the density restriction is area-weighted: it keeps the mass
    fd = 1.0 + rng.random((F * nrad + 1, F * nsec))
    d, _, _ = flux_ref.restrict(fd, fd, fd, surf, F)
    coarse_surf = F * surf[:F * nrad].reshape(nrad, F).sum(axis=1)
    assert np.isclose((d[:nrad] * coarse_surf[:, None]).sum(), (fd[:F * nrad] * surf[:F * nrad, None]).sum())
