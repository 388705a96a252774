"""The 5th-generation tensor-core path (tcgen05) against a CPU product.

fargo_tc_selftest runs one CTA: BF16 operands written to shared memory in the
no-swizzle K-major layout (core matrices of 8 rows x 16 bytes), k / 16
tcgen05.mma.kind::f16 instructions accumulating FP32 in tensor memory, completion
on an mbarrier through tcgen05.commit, and the accumulators read back with
tcgen05.ld.32x32b.  The result must be the exact FP32 product of the BF16 inputs
up to FP32 summation order: small integers make every product and partial sum
exact, so the comparison is bitwise; random operands agree to 1e-5 relative.
"""
import ctypes

import numpy as np
import pytest

from cudaprotoplanetarydisks_gb300 import _capi

pytestmark = pytest.mark.gpu


def bf16_bits(x):
    """BF16 bit patterns of FP32 values (round to nearest even)."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16).astype(np.uint16)
    return r


def bf16_value(bits):
    return (bits.astype(np.uint32) << 16).view(np.float32)


def run(a_bits, b_bits, mode=0):
    lib = _capi.load()
    n, k = b_bits.shape
    d = np.zeros((128, n), dtype=np.float32)
    rc = lib.fargo_tc_selftest(a_bits.ctypes.data, b_bits.ctypes.data, n, k, mode, d.ctypes.data)
    assert rc == 0, rc
    return d


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("n,k", [(64, 16), (64, 64), (16, 32), (128, 128)])
def test_integer_products_are_exact(n, k, mode):
    rng = np.random.default_rng(n * 1000 + k)
    a = rng.integers(-8, 9, size=(128, k)).astype(np.float32)
    b = rng.integers(-8, 9, size=(n, k)).astype(np.float32)
    d = run(bf16_bits(a), bf16_bits(b), mode)
    assert np.array_equal(d, a @ b.T)


def test_descriptor_strides_are_read_as_documented():
    # the descriptor's leading byte offset is the stride along K and the stride
    # byte offset the stride along the rows: with the two fields swapped the
    # product is not the matrix product
    rng = np.random.default_rng(3)
    a = rng.integers(-8, 9, size=(128, 32)).astype(np.float32)
    b = rng.integers(-8, 9, size=(64, 32)).astype(np.float32)
    assert not np.array_equal(run(bf16_bits(a), bf16_bits(b), 2), a @ b.T)


def test_random_products():
    rng = np.random.default_rng(7)
    a = bf16_bits(rng.standard_normal((128, 64)))
    b = bf16_bits(rng.standard_normal((64, 64)))
    d = run(a, b)
    ref = bf16_value(a).astype(np.float64) @ bf16_value(b).astype(np.float64).T
    assert np.abs(d - ref).max() <= 1e-5 * np.abs(ref).max()


@pytest.mark.parametrize("n", [16, 200, 1000, 100003, 196608])
def test_tcgen05_mlp_forward_matches_mma_sync_and_oracle(n):
    # the tcgen05 forward (128-row tiles, accumulators in tensor memory) against the
    # mma.sync forward and the CPU oracle: the same BF16 rounding points, FP32 sums
    # in another order
    import torch
    from cudaprotoplanetarydisks_gb300.learned import MLP, NIN, NOUT, init_params
    from oracle import mlp_ref
    rng = np.random.default_rng(n + 5)
    P = init_params(4)
    P[mlp_ref.OFF_B1:mlp_ref.OFF_W2] = rng.normal(0, 0.1, mlp_ref.NH)
    X = mlp_ref.bf16(rng.normal(0, 1, (n, NIN)))
    m = MLP(max(n, 1024), P)
    xd = torch.tensor(X, dtype=torch.float32).to(torch.bfloat16).cuda()
    ys = {}
    for path in ("mma.sync", "tcgen05"):
        m.set_tensor_path(path)
        yd = torch.full((n, NOUT), float("nan"), dtype=torch.float32, device="cuda")
        m.forward(xd, yd)
        torch.cuda.synchronize()
        m.status()
        ys[path] = yd.cpu().numpy()
    y_ref, _ = mlp_ref.forward(P, X)
    m.close()
    assert np.isfinite(ys["tcgen05"]).all()
    scale = np.linalg.norm(y_ref)
    e_tc = float(np.linalg.norm(ys["tcgen05"] - y_ref) / scale)
    e_ms = float(np.linalg.norm(ys["mma.sync"] - y_ref) / scale)
    d = float(np.linalg.norm(ys["tcgen05"] - ys["mma.sync"]) / scale)
    print(f"n={n}: tcgen05 {e_tc:.2e}, mma.sync {e_ms:.2e} against the oracle; between them {d:.2e}")
    assert e_tc < 1e-3 and d < 1e-3
