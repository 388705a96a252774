"""The FP64 step's divides on the device against IEEE division (numpy).

fdiv64 (the per-cell divides: reciprocal estimate, one Newton step, the quotient
and one correction) must return the correctly rounded quotient except within about
2^-80 of a rounding midpoint, where it may be one ulp off; lim_div (the van Leer
slope limiters: no correction step) must be within about 2^-40 relative.  Outside
|a|, |b| in [2^-500, 2^501) both fall back to IEEE a / b.
"""
import ctypes

import numpy as np
import pytest

from cudaprotoplanetarydisks_gb300 import _capi

pytestmark = pytest.mark.gpu


def _run(a, b):
    lib = _capi.load()
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    q1 = np.empty_like(a)
    q2 = np.empty_like(a)
    P = ctypes.POINTER(ctypes.c_double)
    rc = lib.fargo_div_selftest(a.ctypes.data_as(P), b.ctypes.data_as(P), len(a), q1.ctypes.data_as(P),
                                q2.ctypes.data_as(P))
    assert rc == 0
    return q1, q2


def test_divides_against_ieee():
    rng = np.random.default_rng(7)
    n = 1 << 20
    # operands over the whole range the fields take, and far beyond it
    a = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-140, 140, n)
    b = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-140, 140, n)
    ref = a / b
    q_step, q_lim = _run(a, b)
    ulp = np.spacing(np.abs(ref))
    off = np.abs(q_step - ref)
    assert (off <= ulp).all(), float((off / ulp).max())
    exact = float((off == 0).mean())
    rel = np.abs(q_lim - ref) / np.abs(ref)
    print(f"fdiv64 equal to IEEE on {exact:.6%} of {n} pairs; lim_div max rel error {rel.max():.2e}")
    assert exact > 0.99999
    assert rel.max() < 2.0 ** -37


def test_divides_outside_the_fast_range_are_ieee():
    a = np.array([0.0, -0.0, 1.0, 3.0, 1e-310, 2.0 ** -520, 1e300, 5.0, 7.0, 1.0])
    b = np.array([3.0, 7.0, 1e-310, 2.0 ** -530, 3.0, 5.0, 1e-10, 2.0 ** 510, 1e305, 3.0])
    with np.errstate(over="ignore", divide="ignore"):
        ref = a / b
    q_step, q_lim = _run(a, b)
    # the first four and the out-of-range operands take the IEEE divide: bitwise
    for k in range(9):
        assert q_step[k] == ref[k] or (np.isnan(ref[k]) and np.isnan(q_step[k])), (k, q_step[k], ref[k])
        assert q_lim[k] == ref[k] or (np.isnan(ref[k]) and np.isnan(q_lim[k])), (k, q_lim[k], ref[k])
    assert q_step[9] == ref[9]
    assert abs(q_lim[9] - ref[9]) <= 2.0 ** -37 * abs(ref[9])
