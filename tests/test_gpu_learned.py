"""The stencil MLP's tensor-core kernels against the CPU oracle: forward outputs
and parameter gradients with the kernels' BF16 rounding points, and a training
run that lowers the loss."""
import ctypes

import numpy as np
import pytest
import torch

from cudaprotoplanetarydisks_gb300.learned import MLP, NOUT, NIN, init_params
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("n", [16, 200, 1000, 100003])
def test_forward_and_gradients_match_oracle(n):
    # 100003 rows: many tiles per persistent CTA and a ragged last tile
    rng = np.random.default_rng(n)
    P = init_params(2)
    P[mlp_ref.OFF_B1:mlp_ref.OFF_W2] = rng.normal(0, 0.1, mlp_ref.NH)
    X = mlp_ref.bf16(rng.normal(0, 1, (n, NIN)))
    dy = rng.normal(0, 1, (n, NOUT)).astype(np.float32)
    m = MLP(max(n, 1024), P)
    xd = torch.tensor(X, dtype=torch.float32).to(torch.bfloat16).cuda()
    yd = torch.zeros((n, NOUT), dtype=torch.float32, device="cuda")
    m.forward(xd, yd, train=True)
    m.backward(xd, torch.tensor(dy).cuda())
    torch.cuda.synchronize()
    y_ref, cache = mlp_ref.forward(P, X)
    g_ref = mlp_ref.backward(P, cache, dy)
    ey = rel(yd.cpu().numpy(), y_ref)
    g = m.grad()
    eg = [rel(g[lo:hi], g_ref[lo:hi]) for lo, hi in (
        (mlp_ref.OFF_W1, mlp_ref.OFF_B1), (mlp_ref.OFF_B1, mlp_ref.OFF_W2), (mlp_ref.OFF_W2, mlp_ref.OFF_B2),
        (mlp_ref.OFF_B2, mlp_ref.OFF_W3), (mlp_ref.OFF_W3, mlp_ref.OFF_B3), (mlp_ref.OFF_B3, mlp_ref.NPARAM))]
    print(f"n={n}: y rel {ey:.2e}, gradient rel per block " + " ".join(f"{e:.2e}" for e in eg))
    # BF16 rounding points shared with the oracle; FP32 against FP64 sums and the
    # SFU exponential flip a few roundings (observed at most 8e-5 / 1.2e-4)
    assert ey < 1e-3
    assert max(eg) < 2e-3
    # the padded columns of the last layer get no gradient
    w3 = g[mlp_ref.OFF_W3:mlp_ref.OFF_B3].reshape(mlp_ref.NH, mlp_ref.NOUTP)
    assert not w3[:, NOUT:].any() and not g[mlp_ref.OFF_B3 + NOUT:].any()
    m.close()


def test_backward_is_deterministic():
    rng = np.random.default_rng(8)
    n = 50000
    xd = torch.tensor(rng.normal(0, 1, (n, NIN)), dtype=torch.float32).to(torch.bfloat16).cuda()
    dy = torch.tensor(rng.normal(0, 1, (n, NOUT)), dtype=torch.float32).cuda()
    m = MLP(n, seed=3)
    m.backward(xd, dy)
    g1 = m.grad()
    m.backward(xd, dy)
    assert np.array_equal(g1, m.grad())
    m.close()


def test_misaligned_rows_are_rejected():
    m = MLP(64, seed=0)
    x = torch.zeros((65, NIN), dtype=torch.bfloat16, device="cuda")
    y = torch.zeros((64, NOUT), dtype=torch.float32, device="cuda")
    xv = x.view(-1)[4:4 + 64 * NIN].view(64, NIN)  # 8-byte offset: not 16-byte aligned
    with pytest.raises(RuntimeError):
        m.forward(xv, y)
    m.close()


def test_training_lowers_the_loss():
    rng = np.random.default_rng(11)
    n = 4096
    X = rng.normal(0, 1, (n, NIN))
    target = np.stack([np.tanh(X[:, 0] - 0.5 * X[:, 7]), 0.3 * X[:, 20] * X[:, 21]], axis=1)
    xd = torch.tensor(X, dtype=torch.float32).to(torch.bfloat16).cuda()
    td = torch.tensor(target, dtype=torch.float32).cuda()
    yd = torch.zeros((n, NOUT), dtype=torch.float32, device="cuda")
    m = MLP(n, seed=4)
    losses = []
    for step in range(300):
        m.forward(xd, yd, train=True)
        dy = 2.0 * (yd - td) / n
        losses.append(float(((yd - td) ** 2).sum() / n))
        m.backward(xd, dy)
        m.adam(3e-3)
    torch.cuda.synchronize()
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
    m.close()


# ---------------------------------------------------------------------------
# the correction on coarse disks
import cudaprotoplanetarydisks_gb300 as fg  # noqa: E402
from cudaprotoplanetarydisks_gb300 import learned as L  # noqa: E402


def small_disks(n, seed):
    return fg.c4_disks(n, seed=seed, nrad_choices=(24,))


def test_correction_conserves_mass_and_keeps_density_positive():
    (params, planets), = small_disks(1, 3)
    disk = fg.Disk(params, planets, fg.FARGO_FP32_BULK)
    surf = disk.mesh()[3][:-1]
    m0 = float((disk.field("dens")[:-1] * surf[:, None]).sum())
    corr = L.Correction(L.MLP(params.nrad * params.nsec, seed=9), L.IDENTITY_NORM, 1e-7)
    work = L.workspace(disk)
    for _ in range(2):
        _, accepted = corr.step_DT(disk, work)
        assert accepted
    d = disk.field("dens")[:-1]
    m1 = float((d * surf[:, None]).sum())
    assert d.min() > 0
    # the plain step conserves mass to FP32 roundoff (walls), the correction exactly
    assert abs(m1 - m0) <= 1e-5 * m0
    disk.close()


def test_learned_correction_gains_on_held_out_disks():
    train_disks, held_out = small_disks(4, 11), small_disks(2, 12)
    norm = L.feature_norm(L.generate(train_disks[:1], factor=4, spinup=2, ndt=2))
    tr = L.generate(train_disks, factor=4, spinup=2, ndt=6, norm=norm)
    ho = L.generate(held_out, factor=4, spinup=2, ndt=4, norm=norm)
    scale, var = L.target_stats(tr)
    mlp = L.MLP(24 * 72, seed=1)
    losses = L.train(mlp, tr, scale, var, epochs=40, lr=3e-3)
    assert losses[-1] < losses[0]
    with_net, without = L.evaluate_loss(mlp, ho, scale, var)
    print(f"held-out loss with the network {with_net:.3f}, without {without:.3f}")
    assert with_net < 0.5 * without
    mlp.close()


def test_ring_neutral_correction_keeps_every_ring_mass():
    rng = np.random.default_rng(21)
    nrad, nsec = 12, 40
    n = nrad * nsec
    y = torch.tensor(rng.normal(0, 1, (n, NOUT)), dtype=torch.float32, device="cuda")
    y_ref = y.cpu().numpy().astype(np.float64)
    L.ring_center(y, nrad, nsec)
    yr = y_ref[:, 0].reshape(nrad, nsec)
    expect = (yr - yr.mean(axis=1, keepdims=True)).ravel()
    assert np.allclose(y.cpu().numpy()[:, 0], expect, atol=1e-6)
    assert np.array_equal(y.cpu().numpy()[:, 1], y_ref[:, 1].astype(np.float32))
    # the divergence of ring-neutral outputs moves no mass between rings
    surf = torch.tensor(np.linspace(1e-3, 4e-3, nrad + 1), dtype=torch.float64, device="cuda")
    ds = torch.empty(n, dtype=torch.float32, device="cuda")
    rc = L._capi.load().fargo_learned_divergence(ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(surf.data_ptr()),
                                                 nrad, nsec, ctypes.c_float(1.0), ctypes.c_void_p(ds.data_ptr()),
                                                 None)
    assert rc == 0
    torch.cuda.synchronize()
    ring_dm = (ds.cpu().numpy().astype(np.float64).reshape(nrad, nsec)).sum(axis=1)
    assert np.abs(ring_dm).max() < 1e-4, np.abs(ring_dm).max()


def test_limited_correction_keeps_density_positive_and_mass():
    (params, planets), = small_disks(1, 5)
    disk = fg.Disk(params, planets, fg.FARGO_FP32_BULK)
    disk.step_DT()
    nrad, nsec = params.nrad, params.nsec
    n = nrad * nsec
    surf = disk.mesh()[3]
    surf_d = torch.tensor(surf, dtype=torch.float64, device="cuda")
    dens = disk.field("dens")[:-1].astype(np.float64)
    rng = np.random.default_rng(2)
    y = torch.tensor(rng.normal(0, 1, (n, NOUT)), dtype=torch.float32, device="cuda")
    lib = L._capi.load()
    plain = torch.empty(n, dtype=torch.float32, device="cuda")
    lim = torch.empty(n, dtype=torch.float32, device="cuda")
    beta = 0.5
    for scale, big in ((float(dens.mean()), True), (1e-7 * float(dens.mean()), False)):
        assert lib.fargo_learned_divergence(ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(surf_d.data_ptr()), nrad,
                                            nsec, ctypes.c_float(scale), ctypes.c_void_p(plain.data_ptr()), None) == 0
        assert lib.fargo_learned_divergence_limited(disk.h, ctypes.c_void_p(y.data_ptr()), ctypes.c_float(scale),
                                                    ctypes.c_float(beta), ctypes.c_void_p(lim.data_ptr())) == 0
        torch.cuda.synchronize()
        dp = plain.cpu().numpy().astype(np.float64).reshape(nrad, nsec)
        dl = lim.cpu().numpy().astype(np.float64).reshape(nrad, nsec)
        mass_l = (dl * surf[:nrad, None]).sum()
        assert abs(mass_l) <= 1e-5 * (np.abs(dl) * surf[:nrad, None]).sum()
        assert (dens + dl >= (1.0 - beta) * dens * (1.0 - 1e-5)).all()
        if big:
            assert (dens + dp < 0).any()  # the unlimited correction would empty cells
        else:
            assert np.allclose(dl, dp, rtol=1e-5, atol=1e-12 * float(dens.mean()))
    disk.close()


@pytest.mark.parametrize("prec", [fg.FARGO_FP32_BULK, fg.FARGO_FP64])
def test_features_match_oracle(prec):
    import math

    from oracle import features_ref
    (params, planets), = small_disks(1, 7)
    disk = fg.Disk(params, planets, prec)
    disk.step_DT()
    n = params.nrad * params.nsec
    x = torch.empty((n, NIN), dtype=torch.bfloat16, device="cuda")
    L.Correction(None, L.IDENTITY_NORM, 1.0).features(disk, x)
    got = x.float().cpu().numpy().astype(np.float64)
    p = disk.planets()[0]
    ref = features_ref.features(disk.field("dens"), disk.field("vrad"), disk.field("vtheta"), disk.mesh()[1],
                                math.atan2(p.y, p.x))
    disk.close()
    assert not got[:, 125:].any()
    diff = np.abs(got - ref)[:, :125].reshape(n, 25, 5)
    # the azimuth channel wraps at +-1: a cell at the wrap point may land on either side
    diff[:, :, 4] = np.minimum(diff[:, :, 4], np.abs(diff[:, :, 4] - 2.0))
    r = np.abs(ref)[:, :125].reshape(n, 25, 5)
    # BF16 output (relative half-ulp 2^-9; a rounding flip from the FP32 arithmetic
    # gives one ulp, 2^-8), plus the FP32 arithmetic's absolute error per channel
    atol = np.array([1e-9, 1e-9, 2e-6, 1e-6, 1e-6])
    assert (diff <= 2.0 ** -7 * r + atol).all(), float((diff - 2.0 ** -7 * r).max())


def test_divergence_loss_and_adjoint_match_oracle():
    from oracle import flux_ref
    rng = np.random.default_rng(31)
    nrad, nsec, scale, inv_var = 20, 60, 0.37, 2.5
    n = nrad * nsec
    surf = np.linspace(1e-3, 5e-3, nrad + 1)
    y = rng.normal(0, 1, (n, NOUT)).astype(np.float32)
    target = rng.normal(0, 1, n).astype(np.float32)
    ds_ref, loss_ref, dy_ref = flux_ref.loss(y, target, surf, nrad, nsec, scale, inv_var)
    buf = L._buffers(n)
    L._loss_call(L._capi.load(), torch.tensor(y).cuda(), torch.tensor(target).cuda(),
                 torch.tensor(surf, dtype=torch.float64).cuda(), nrad, nsec, scale, inv_var, buf)
    torch.cuda.synchronize()
    ds, dy, lo = buf[0].cpu().numpy(), buf[2].cpu().numpy(), float(buf[4].item())
    # FP32 kernels against FP64: a few ulps per value
    assert rel(ds, ds_ref) < 1e-6
    assert abs(lo - loss_ref) < 1e-5 * loss_ref
    assert rel(dy, dy_ref) < 1e-5


@pytest.mark.parametrize("prec,tol", [(fg.FARGO_FP64, 1e-13), (fg.FARGO_FP32_BULK, 2e-7)])
def test_restriction_matches_oracle(prec, tol):
    from oracle import flux_ref
    (params, planets), = fg.c4_disks(1, seed=13, nrad_choices=(12,))
    fine = fg.Disk(L.fine_params(params, 4), planets, prec)
    fine.step_DT()
    coarse = fg.Disk(params, planets, prec)
    L.restrict(fine, coarse, 4)
    ref = flux_ref.restrict(fine.field("dens"), fine.field("vrad"), fine.field("vtheta"), fine.mesh()[3], 4)
    for name, r in zip(("dens", "vrad", "vtheta"), ref):
        got = coarse.field(name)
        assert got.shape == r.shape
        assert np.abs(got - r).max() <= tol * np.abs(r).max(), (name, float(np.abs(got - r).max()))
    fine.close()
    coarse.close()
