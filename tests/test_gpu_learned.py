"""The stencil MLP's tensor-core kernels against the CPU oracle: forward outputs
and parameter gradients with the kernels' BF16 rounding points, and a training
run that lowers the loss."""
import numpy as np
import pytest
import torch

from cudaprotoplanetarydisks_gb300.learned import MLP, NOUT, NIN, init_params
from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("n", [16, 200, 1000])
def test_forward_and_gradients_match_oracle(n):
    rng = np.random.default_rng(n)
    P = init_params(2)
    P[mlp_ref.OFF_B1:mlp_ref.OFF_W2] = rng.normal(0, 0.1, mlp_ref.NH)
    X = mlp_ref.bf16(rng.normal(0, 1, (n, NIN)))
    dy = rng.normal(0, 1, (n, NOUT)).astype(np.float32)
    m = MLP(1024, P)
    xd = torch.tensor(X, dtype=torch.float32).to(torch.bfloat16).cuda()
    yd = torch.zeros((n, NOUT), dtype=torch.float32, device="cuda")
    m.forward(xd, yd, train=True)
    m.backward(xd, torch.tensor(dy).cuda())
    torch.cuda.synchronize()
    y_ref, cache = mlp_ref.forward(P, X)
    g_ref = mlp_ref.backward(P, cache, dy)
    assert rel(yd.cpu().numpy(), y_ref) < 1e-2
    g = m.grad()
    for lo, hi in ((mlp_ref.OFF_W1, mlp_ref.OFF_B1), (mlp_ref.OFF_B1, mlp_ref.OFF_W2), (mlp_ref.OFF_W2, mlp_ref.OFF_B2),
                   (mlp_ref.OFF_B2, mlp_ref.OFF_W3), (mlp_ref.OFF_W3, mlp_ref.OFF_B3), (mlp_ref.OFF_B3, mlp_ref.NPARAM)):
        assert rel(g[lo:hi], g_ref[lo:hi]) < 3e-2, (lo, hi)
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
